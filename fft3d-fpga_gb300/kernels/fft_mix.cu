// fft_mix.cu - the complex instantiations of the mixed-radix axis kernel
// (kernels/fft_mix_impl.cuh), its launch shape and the choice of radices.
#include "fft_mix_impl.cuh"

namespace fftgb {

namespace {
MixFn g_mix[2][2][2];  // [inverse][strided][more than 256 threads]
MixPairTable g_mix2 = {};  // two-stage kernels
MixTripleTable g_mix3 = {};  // three-stage kernels
MixPairEpiTable g_mix2_epi = {};  // four-step passes, two-stage kernels
MixEpiTable g_mix_epi = {};       // four-step passes, generic kernels
MixTripleEpiTable g_mix3_epi = {};  // four-step passes, three-stage kernels
constexpr int MIX_SMEM_MAX = 100 * 1024;
bool g_mix_ready = false;

int env_int_mix(const char *name) {
  const char *e = getenv(name);
  return (e && *e) ? atoi(e) : 0;
}
}  // namespace

cudaError_t mix_kernels_init() {
  if (g_mix_ready) return cudaSuccess;
  g_mix[0][0][0] = k_mix<false, false, 256>;
  g_mix[1][0][0] = k_mix<true, false, 256>;
  g_mix[0][1][0] = k_mix<false, true, 256>;
  g_mix[1][1][0] = k_mix<true, true, 256>;
  g_mix[0][0][1] = k_mix<false, false, MIX_THREADS>;
  g_mix[1][0][1] = k_mix<true, false, MIX_THREADS>;
  g_mix[0][1][1] = k_mix<false, true, MIX_THREADS>;
  g_mix[1][1][1] = k_mix<true, true, MIX_THREADS>;
  for (int d = 0; d < 2; d++)
    for (int st = 0; st < 2; st++)
      for (int big = 0; big < 2; big++) {
        const cudaError_t e = cudaFuncSetAttribute(
            (const void *)g_mix[d][st][big], cudaFuncAttributeMaxDynamicSharedMemorySize,
            MIX_SMEM_MAX);
        if (e != cudaSuccess) return e;
      }
  mix2_fill_a(g_mix2);
  mix2_fill_b(g_mix2);
  mix2_fill_c(g_mix2);
  for (int r0 = 0; r0 < 11; r0++)
    for (int r1 = 0; r1 < 11; r1++)
      for (int d = 0; d < 2; d++)
        for (int st = 0; st < 2; st++) {
          MixFn f = g_mix2[r0][r1][d][st];
          if (!f) continue;
          const cudaError_t e = cudaFuncSetAttribute(
              (const void *)f, cudaFuncAttributeMaxDynamicSharedMemorySize, MIX_SMEM_MAX);
          if (e != cudaSuccess) return e;
        }
  mix3_fill_d(g_mix3);
  mix3_fill_e(g_mix3);
  mix3_fill_f(g_mix3);
  mix3_fill_g(g_mix3);
  mix3_fill_h(g_mix3);
  mix3_fill_i(g_mix3);
  for (int r0 = 0; r0 < 11; r0++)
    for (int r1 = 0; r1 < 11; r1++)
      for (int r2 = 0; r2 < 11; r2++)
        for (int d = 0; d < 2; d++)
          for (int st = 0; st < 2; st++) {
            MixFn f = g_mix3[r0][r1][r2][d][st];
            if (!f) continue;
            const cudaError_t e = cudaFuncSetAttribute(
                (const void *)f, cudaFuncAttributeMaxDynamicSharedMemorySize, MIX_SMEM_MAX);
            if (e != cudaSuccess) return e;
          }
  mix2_fill_epi_a(g_mix2_epi);
  mix2_fill_epi_b(g_mix2_epi);
  mix2_fill_epi_c(g_mix2_epi);
  mix_fill_epi(g_mix_epi);
  mix3_fill_epi_d(g_mix3_epi);
  mix3_fill_epi_e(g_mix3_epi);
  mix3_fill_epi_f(g_mix3_epi);
  mix3_fill_epi_g(g_mix3_epi);
  mix3_fill_epi_h(g_mix3_epi);
  mix3_fill_epi_i(g_mix3_epi);
  for (int r0 = 0; r0 < 11; r0++)
    for (int r1 = 0; r1 < 11; r1++)
      for (int r2 = 0; r2 < 11; r2++)
        for (int ep = 0; ep < 2; ep++)
          for (int d = 0; d < 2; d++) {
            MixFn f = g_mix3_epi[r0][r1][r2][ep][d];
            if (!f) continue;
            const cudaError_t e = cudaFuncSetAttribute(
                (const void *)f, cudaFuncAttributeMaxDynamicSharedMemorySize, MIX_SMEM_MAX);
            if (e != cudaSuccess) return e;
          }
  for (int r0 = 0; r0 < 11; r0++)
    for (int r1 = 0; r1 < 11; r1++)
      for (int ep = 0; ep < 2; ep++)
        for (int d = 0; d < 2; d++) {
          MixFn f = g_mix2_epi[r0][r1][ep][d];
          if (!f) continue;
          const cudaError_t e = cudaFuncSetAttribute(
              (const void *)f, cudaFuncAttributeMaxDynamicSharedMemorySize, MIX_SMEM_MAX);
          if (e != cudaSuccess) return e;
        }
  for (int ep = 0; ep < 2; ep++)
    for (int d = 0; d < 2; d++)
      for (int big = 0; big < 2; big++) {
        const cudaError_t e = cudaFuncSetAttribute((const void *)g_mix_epi[ep][d][big],
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   MIX_SMEM_MAX);
        if (e != cudaSuccess) return e;
      }
  const cudaError_t e = mix_real_init();
  if (e != cudaSuccess) return e;
  g_mix_ready = true;
  return cudaSuccess;
}

namespace {
const int kMixRad[11] = {16, 15, 12, 10, 9, 8, 6, 5, 4, 3, 2};  // the kernel's stage order
const int kMixExp[11][3] = {{4, 0, 0}, {0, 1, 1}, {2, 1, 0}, {1, 0, 1}, {0, 2, 0}, {3, 0, 0},
                            {1, 1, 0}, {0, 0, 1}, {2, 0, 0}, {0, 1, 0}, {1, 0, 0}};

// Threads per line that a factorisation needs with the butterflies per thread
// of the small (big = false) or the 512-thread CTAs.
int mix_threads(int n, const int *rad, int nst, bool big) {
  int t = 1;
  for (int i = 0; i < nst; i++) {
    const int m = n / rad[i], nb = mix_nb(rad[i], big);
    const int ti = (m + nb - 1) / nb;
    if (ti > t) t = ti;
  }
  return t;
}

struct MixSearch {
  int n;
  int cur[MIX_MAXST], ncur;
  int best[MIX_MAXST], nbest;
  long long best_score;
  bool simple;  // radices 16, 8, 4, 2, 5, 3 only
  void leaf() {
    const bool small = mix_threads(n, cur, ncur, false) <= MIX_SMALL;
    const int t = mix_threads(n, cur, ncur, !small);
    // fewer stages first (the 512-thread CTAs count one more), then the
    // small CTAs, then fewer threads per line
    const long long score = ((long long)(ncur + (small ? 0 : 1)) * 2 + (small ? 0 : 1)) * 100000 + t;
    if (best_score < 0 || score < best_score) {
      best_score = score;
      nbest = ncur;
      for (int i = 0; i < ncur; i++) best[i] = cur[i];
    }
  }
  void dfs(int ri, int e2, int e3, int e5) {
    if (e2 == 0 && e3 == 0 && e5 == 0) {
      leaf();
      return;
    }
    if (ri >= 11 || ncur >= MIX_MAXST) return;
    const int r = kMixRad[ri];
    const bool allowed = !simple || r == 16 || r == 8 || r == 4 || r == 2 || r == 5 || r == 3;
    const int *x = kMixExp[ri];
    // take k stages of radix r (as many as fit first), then the next radix
    int k = 0;
    if (allowed)
      while ((k + 1) * x[0] <= e2 && (k + 1) * x[1] <= e3 && (k + 1) * x[2] <= e5 &&
             ncur + k + 1 <= MIX_MAXST)
        k++;
    for (; k >= 0; k--) {
      for (int i = 0; i < k; i++) cur[ncur + i] = r;
      ncur += k;
      dfs(ri + 1, e2 - k * x[0], e3 - k * x[1], e5 - k * x[2]);
      ncur -= k;
    }
  }
};
}  // namespace

int mix_radices(int n, int *rad, bool simple) {
  if (n < 2 || n > MIX_MAXN) return 0;
  int a = 0, b = 0, c = 0, r = n;
  while (r % 2 == 0) { r /= 2; a++; }
  while (r % 3 == 0) { r /= 3; b++; }
  while (r % 5 == 0) { r /= 5; c++; }
  if (r != 1) return 0;
  MixSearch ms;
  ms.n = n;
  ms.ncur = 0;
  ms.nbest = 0;
  ms.best_score = -1;
  ms.simple = simple;
  ms.dfs(0, a, b, c);
  if (ms.nbest < 1 || mix_threads(n, ms.best, ms.nbest, true) > MIX_THREADS) return 0;
  for (int i = 0; i < ms.nbest; i++) rad[i] = ms.best[i];
  return ms.nbest;
}

static int gcd_int(int x, int y) {
  while (y) {
    const int t = x % y;
    x = y;
    y = t;
  }
  return x;
}

cudaError_t mix_shape(const MixArgs &a, int lines_per_cta, bool real, MixShape *sh) {
  if (a.n < 2 || a.n > MIX_MAXN || a.nst < 1 || a.nst > MIX_MAXST || a.nlines < 1 ||
      a.inner < 1 || (real && a.inner != 1))
    return cudaErrorInvalidValue;
  // radices grouped in the kernel's stage order
  long long prod = 1;
  int prev = 0;
  unsigned long long code = 0;
  for (int i = 0; i < a.nst; i++) {
    const int rank = mix_rank(a.rad[i]);
    if (rank < prev) return cudaErrorInvalidValue;
    prev = rank;
    prod *= a.rad[i];
    code |= (unsigned long long)rank << (4 * i);
  }
  if (prod != a.n) return cudaErrorInvalidValue;
  const bool strided = a.inner > 1;
  const int n = a.n;
  // threads per line, at least: the small CTAs where one line fits them
  const int ts = mix_threads(n, a.rad, a.nst, false);
  const bool big = ts > MIX_SMALL;
  const int t0 = big ? mix_threads(n, a.rad, a.nst, true) : ts;
  if (t0 > MIX_THREADS) return cudaErrorInvalidValue;
  int ptarget = env_int_mix("FFTGB_MIX_PTS");
  if (ptarget <= 0) ptarget = strided ? 8192 : 4096;
  const int cap = big ? MIX_THREADS : MIX_SMALL;
  int F = lines_per_cta > 0 ? lines_per_cta : env_int_mix("FFTGB_MIX_F");
  if (F <= 0) {
    F = 1;
    while (2LL * F * n <= ptarget && 2 * F * t0 <= cap) F *= 2;
  }
  if ((long long)F > a.nlines) {
    int f = 1;
    while (2LL * f <= a.nlines) f *= 2;
    F = f;
  }
  // F*T a multiple of the warp where that fits the cap (always for the
  // power-of-two F chosen above), else the fewest threads per line
  const int g = 32 / gcd_int(F, 32);
  int T = (t0 + g - 1) / g * g;
  if ((long long)F * T > cap) T = t0;
  if ((long long)F * T > cap) return cudaErrorInvalidConfiguration;
  const long long smem = strided ? (long long)n * F * 8 : (long long)F * (n + (n >> 4) + 1) * 8;
  if ((a.nst > 1 || real) && smem > MIX_SMEM_MAX) return cudaErrorInvalidConfiguration;
  const long long grid = (a.nlines + F - 1) / F;
  if (grid > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  sh->F = F;
  sh->T = T;
  sh->big = big;
  sh->grid = grid;
  sh->smem = (a.nst > 1 || real) ? (size_t)smem : 0;
  sh->rcode = code;
  return cudaSuccess;
}

cudaError_t launch_mix(int inverse, const MixArgs &a, cudaStream_t s, int lines_per_cta) {
  if (!g_mix_ready) return cudaErrorInvalidValue;
  MixShape sh;
  const cudaError_t e = mix_shape(a, lines_per_cta, false, &sh);
  if (e != cudaSuccess) return e;
  const int d = inverse ? 1 : 0, st = a.inner > 1 ? 1 : 0;
  MixFn f = g_mix[d][st][sh.big ? 1 : 0];
  if (a.epi) {  // a four-step pass
    if (a.epi > 2 || (a.epi == 1 && (a.inner < 2 || !a.tw_lo || !a.tw_hi)) ||
        (a.epi == 2 && (a.inner != 1 || a.ep_n2 < 1 || a.ep_N < a.ep_n2)))
      return cudaErrorInvalidValue;
    f = g_mix_epi[a.epi - 1][d][sh.big ? 1 : 0];
    if (!sh.big && env_int_mix("FFTGB_MIX_GENERIC") != 1) {
      MixFn fs = nullptr;
      if (a.nst == 2) fs = g_mix2_epi[mix_rank(a.rad[0])][mix_rank(a.rad[1])][a.epi - 1][d];
      if (a.nst == 3)
        fs = g_mix3_epi[mix_rank(a.rad[0])][mix_rank(a.rad[1])][mix_rank(a.rad[2])][a.epi - 1][d];
      if (fs) f = fs;
    }
  } else if (!sh.big && env_int_mix("FFTGB_MIX_GENERIC") != 1) {
    MixFn fs = nullptr;
    if (a.nst == 2) fs = g_mix2[mix_rank(a.rad[0])][mix_rank(a.rad[1])][d][st];
    if (a.nst == 3) fs = g_mix3[mix_rank(a.rad[0])][mix_rank(a.rad[1])][mix_rank(a.rad[2])][d][st];
    if (fs) f = fs;
  }
  MixArgs b = a;
  b.rcode = sh.rcode;
  f<<<(unsigned)sh.grid, sh.F * sh.T, sh.smem, s>>>(b, sh.F, sh.T);
  return cudaGetLastError();
}

}  // namespace fftgb
