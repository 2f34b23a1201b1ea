// fft_mix.cu - FFTs of length n = 2^a 3^b 5^c (n <= 8192) along one axis,
// one kernel per axis: a mixed-radix Stockham transform with radix-16, 8, 4,
// 2, 5 and 3 stages.  The reference supports powers of two only; this is
// the non-power-of-two extension for the smooth lengths (any other length
// takes Bluestein's algorithm, fft_blue.cu).
//
// Stage s of radix R (NS = product of the earlier radices, m = n/R) takes,
// for every butterfly j < m with k = j mod NS, the points j + q*m (q < R),
// multiplies point q by W_n^(q*k*n/(NS*R)), applies the R-point DFT and
// writes output q to (j - k)*R + k + q*NS.  After the last stage the line is
// in natural order.  The twiddle exponent q*k*n/(NS*R) is an exact integer
// below n, so every twiddle is one entry of a FP64-generated table of n
// values.  k = j mod NS comes from a multiply-high by ceil(2^32/NS), exact
// because j*NS < 2^32 (Granlund and Montgomery, "Division by invariant
// integers using multiplication", PLDI 1994).
//
// The first stage reads its points straight from global memory and the last
// writes straight to it (both at consecutive j, so consecutive threads touch
// consecutive points of a line, or consecutive lines of a strided axis);
// the stages in between go through one shared-memory copy of the CTA's lines.
// Each thread owns butterflies t, t + T, ... of every stage (T threads per
// line, T >= n/16, so at most ceil(16/R) butterflies of radix R): it reads all
// of them into registers, the CTA synchronises, and it writes them back, so
// one buffer serves every stage in place.  The inverse transform is the
// forward one between two real/imaginary swaps.
//
// Contiguous lines (stride 1) sit one after the other in shared memory with
// one pad point per 16 (the radix-R write of the first stage goes at stride
// R); lines of a strided axis are interleaved point by point ([point][line]),
// so a warp reading one point of consecutive lines reads one run.
#include "fft_core.cuh"
#include "fft_mix.cuh"

namespace fftgb {

// Exact values of the radix-3 and radix-5 DFT constants (mathematical
// constants).
#define FFTGB_S3 0.86602540378443864676f   // sin(2 pi/3) = sqrt(3)/2
#define FFTGB_C5A 0.30901699437494742410f  // cos(2 pi/5)
#define FFTGB_C5B 0.80901699437494742410f  // -cos(4 pi/5)
#define FFTGB_S5A 0.95105651629515357212f  // sin(2 pi/5)
#define FFTGB_S5B 0.58778525229247312917f  // sin(4 pi/5)

template <int R>
__device__ __forceinline__ void dftm(float2 *v) {
  dft<R>(v);
}

template <>
__device__ __forceinline__ void dftm<3>(float2 *v) {
  const float2 a = v[0], t = cadd(v[1], v[2]), d = csub(v[1], v[2]);
  const float2 m = make_float2(a.x - 0.5f * t.x, a.y - 0.5f * t.y);
  const float2 r = make_float2(FFTGB_S3 * d.y, -FFTGB_S3 * d.x);  // -i sin(2pi/3) d
  v[0] = cadd(a, t);
  v[1] = cadd(m, r);
  v[2] = csub(m, r);
}

template <>
__device__ __forceinline__ void dftm<5>(float2 *v) {
  const float2 x0 = v[0];
  const float2 t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
  const float2 d1 = csub(v[1], v[4]), d2 = csub(v[2], v[3]);
  const float2 a1 = make_float2(x0.x + FFTGB_C5A * t1.x - FFTGB_C5B * t2.x,
                                x0.y + FFTGB_C5A * t1.y - FFTGB_C5B * t2.y);
  const float2 a2 = make_float2(x0.x - FFTGB_C5B * t1.x + FFTGB_C5A * t2.x,
                                x0.y - FFTGB_C5B * t1.y + FFTGB_C5A * t2.y);
  const float2 b1 = make_float2(FFTGB_S5A * d1.x + FFTGB_S5B * d2.x,
                                FFTGB_S5A * d1.y + FFTGB_S5B * d2.y);
  const float2 b2 = make_float2(FFTGB_S5B * d1.x - FFTGB_S5A * d2.x,
                                FFTGB_S5B * d1.y - FFTGB_S5A * d2.y);
  const float2 r1 = cmul_mi(b1), r2 = cmul_mi(b2);  // -i b
  v[0] = make_float2(x0.x + t1.x + t2.x, x0.y + t1.y + t2.y);
  v[1] = cadd(a1, r1);
  v[4] = csub(a1, r1);
  v[2] = cadd(a2, r2);
  v[3] = csub(a2, r2);
}

constexpr int MIX_EMAX = 16;      // points per thread and stage, at most
constexpr int MIX_THREADS = 512;  // threads per CTA, at most

struct MixLine {
  long long gbase;  // global index of the line's point 0
  int fl;           // line within the CTA
  int t;            // thread within the line
  int T;            // threads per line
  int F;            // lines per CTA
  bool ok;          // the line exists
};

template <bool STRIDED>
__device__ __forceinline__ int mix_sidx(const MixLine &L, int lp, int i) {
  return STRIDED ? i * L.F + L.fl : L.fl * lp + i + (i >> 4);
}

// One stage.  MODE 0: the first (global -> shared), 1: a middle one
// (shared -> shared), 2: the last (shared -> global), 3: the only one
// (global -> global).
template <int R, int MODE, bool INV, bool STRIDED>
__device__ __forceinline__ void mix_stage(const MixArgs &a, const MixLine &L, float2 *sm,
                                          int lp, int ns) {
  constexpr bool FIRST = MODE == 0 || MODE == 3, LAST = MODE >= 2;
  constexpr int NB = (MIX_EMAX + R - 1) / R;
  const int n = a.n, m = n / R;
  const int tws = n / (ns * R);
  const unsigned magic = ns > 1 ? 0xffffffffu / (unsigned)ns + 1u : 0u;
  const long long gstride = STRIDED ? a.inner : 1;
  float2 v[NB][R];
#pragma unroll
  for (int b = 0; b < NB; b++) {
    const int j = L.t + b * L.T;
    if (j < m) {
      if (FIRST) {
        const float2 *src = a.in + L.gbase + (long long)j * gstride;
#pragma unroll
        for (int q = 0; q < R; q++) {
          float2 x = make_float2(0.f, 0.f);
          if (L.ok) x = src[(long long)(q * m) * gstride];
          v[b][q] = INV ? cswap(x) : x;
        }
      } else {
        const int k = j - (int)__umulhi((unsigned)j, magic) * ns;
#pragma unroll
        for (int q = 0; q < R; q++) v[b][q] = sm[mix_sidx<STRIDED>(L, lp, j + q * m)];
        const int kt = k * tws;
#pragma unroll
        for (int q = 1; q < R; q++) v[b][q] = cmul(v[b][q], __ldg(&a.w[q * kt]));
      }
      dftm<R>(v[b]);
    }
  }
  // every read of this stage lands before any write of it (one buffer)
  if (MODE == 1) __syncthreads();
#pragma unroll
  for (int b = 0; b < NB; b++) {
    const int j = L.t + b * L.T;
    if (j < m) {
      const int k = FIRST ? 0 : j - (int)__umulhi((unsigned)j, magic) * ns;
      const int d = (j - k) * R + k;
      if (LAST) {
        if (L.ok) {
          float2 *dst = a.out + L.gbase + (long long)d * gstride;
#pragma unroll
          for (int q = 0; q < R; q++) {
            float2 y = INV ? cswap(v[b][q]) : v[b][q];
            if (a.scale != 1.0f) y = cscale(y, a.scale);
            dst[(long long)(q * ns) * gstride] = y;
          }
        }
      } else {
#pragma unroll
        for (int q = 0; q < R; q++) sm[mix_sidx<STRIDED>(L, lp, d + q * ns)] = v[b][q];
      }
    }
  }
  if (!LAST) __syncthreads();
}

template <int MODE, bool INV, bool STRIDED>
__device__ __forceinline__ void mix_stage_r(int r, const MixArgs &a, const MixLine &L,
                                            float2 *sm, int lp, int ns) {
  switch (r) {
    case 16: mix_stage<16, MODE, INV, STRIDED>(a, L, sm, lp, ns); break;
    case 8: mix_stage<8, MODE, INV, STRIDED>(a, L, sm, lp, ns); break;
    case 4: mix_stage<4, MODE, INV, STRIDED>(a, L, sm, lp, ns); break;
    case 2: mix_stage<2, MODE, INV, STRIDED>(a, L, sm, lp, ns); break;
    case 5: mix_stage<5, MODE, INV, STRIDED>(a, L, sm, lp, ns); break;
    default: mix_stage<3, MODE, INV, STRIDED>(a, L, sm, lp, ns); break;
  }
}

// NT: the most threads a CTA of the instantiation has; CTAs of up to 256
// threads run three to an SM (80 registers), larger ones one (128).
template <bool INV, bool STRIDED, int NT>
__global__ void __launch_bounds__(NT, NT <= 256 ? 3 : 1) k_mix(const MixArgs a, int F, int T) {
  extern __shared__ float2 smem[];
  const int tid = threadIdx.x;
  MixLine L;
  L.F = F;
  L.T = T;
  L.fl = STRIDED ? tid % F : tid / T;
  L.t = STRIDED ? tid / F : tid % T;
  const long long line = (long long)blockIdx.x * F + L.fl;
  L.ok = line < a.nlines;
  L.gbase = 0;
  if (L.ok) {
    const long long o = line / a.inner;
    L.gbase = o * a.n * a.inner + (line - o * a.inner);
  }
  const int lp = a.n + (a.n >> 4) + 1;  // contiguous layout: padded line pitch
  const int nst = a.nst;
  if (nst == 1) {
    mix_stage_r<3, INV, STRIDED>(a.rad[0], a, L, smem, lp, 1);
    return;
  }
  mix_stage_r<0, INV, STRIDED>(a.rad[0], a, L, smem, lp, 1);
  // The middle stages, one loop per radix (the radices come grouped in the
  // order 16, 8, 4, 2, 5, 3): each loop holds one stage body, so what the
  // compiler hoists out of it belongs to that radix alone.
  int ns = a.rad[0], st = 1;
#define FFTGB_MIX_MID(R)                                   \
  for (; st < nst - 1 && a.rad[st] == R; st++) {           \
    mix_stage<R, 1, INV, STRIDED>(a, L, smem, lp, ns);     \
    ns *= R;                                               \
  }
  FFTGB_MIX_MID(16)
  FFTGB_MIX_MID(8)
  FFTGB_MIX_MID(4)
  FFTGB_MIX_MID(2)
  FFTGB_MIX_MID(5)
  FFTGB_MIX_MID(3)
#undef FFTGB_MIX_MID
  mix_stage_r<2, INV, STRIDED>(a.rad[nst - 1], a, L, smem, lp, ns);
}

namespace {
typedef void (*MixFn)(const MixArgs, int, int);
MixFn g_mix[2][2][2];  // [inverse][strided][more than 256 threads]
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
  g_mix_ready = true;
  return cudaSuccess;
}

int mix_radices(int n, int *rad) {
  if (n < 2 || n > MIX_MAXN) return 0;
  int a = 0, b = 0, c = 0, r = n;
  while (r % 2 == 0) { r /= 2; a++; }
  while (r % 3 == 0) { r /= 3; b++; }
  while (r % 5 == 0) { r /= 5; c++; }
  if (r != 1) return 0;
  int ns = 0, n16 = a / 4;
  const int rem = a % 4;
  int low[2] = {0, 0}, nlow = 0;
  if (rem == 1 && n16 > 0) {
    n16--;
    low[nlow++] = 8;
    low[nlow++] = 4;
  } else if (rem) {
    low[nlow++] = 1 << rem;
  }
  for (int i = 0; i < n16; i++) rad[ns++] = 16;
  for (int i = 0; i < nlow; i++) rad[ns++] = low[i];
  for (int i = 0; i < c; i++) rad[ns++] = 5;
  for (int i = 0; i < b; i++) rad[ns++] = 3;
  return ns <= MIX_MAXST ? ns : 0;
}

static int gcd_int(int x, int y) {
  while (y) {
    const int t = x % y;
    x = y;
    y = t;
  }
  return x;
}

cudaError_t launch_mix(int inverse, const MixArgs &a, cudaStream_t s, int lines_per_cta) {
  if (!g_mix_ready || a.n < 2 || a.n > MIX_MAXN || a.nst < 1 || a.nst > MIX_MAXST ||
      a.nlines < 1 || a.inner < 1)
    return cudaErrorInvalidValue;
  // radices grouped in the order 16, 8, 4, 2, 5, 3 (the kernel's middle loops)
  long long prod = 1;
  int prev = 0;
  for (int i = 0; i < a.nst; i++) {
    const int r = a.rad[i];
    const int rank = r == 16 ? 0 : r == 8 ? 1 : r == 4 ? 2 : r == 2 ? 3 : r == 5 ? 4 : r == 3 ? 5 : -1;
    if (rank < prev) return cudaErrorInvalidValue;
    prev = rank;
    prod *= r;
  }
  if (prod != a.n) return cudaErrorInvalidValue;
  const bool strided = a.inner > 1;
  const int n = a.n;
  const int t0 = (n + MIX_EMAX - 1) / MIX_EMAX;  // threads per line, at least
  int ptarget = env_int_mix("FFTGB_MIX_PTS");
  if (ptarget <= 0) ptarget = strided ? 8192 : 4096;
  // CTAs of at most 256 threads (three per SM) unless one line needs more
  const int cap = t0 > 256 ? MIX_THREADS : 256;
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
  const int g = 32 / gcd_int(F, 32);
  const int T = (t0 + g - 1) / g * g;  // F*T a multiple of the warp where it can be
  if ((long long)F * T > MIX_THREADS) return cudaErrorInvalidConfiguration;
  const long long smem = strided ? (long long)n * F * 8 : (long long)F * (n + (n >> 4) + 1) * 8;
  if (a.nst > 1 && smem > MIX_SMEM_MAX) return cudaErrorInvalidConfiguration;
  const long long grid = (a.nlines + F - 1) / F;
  if (grid > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  const int big = F * T > 256 ? 1 : 0;
  g_mix[inverse ? 1 : 0][strided ? 1 : 0][big]<<<(unsigned)grid, F * T,
                                                  a.nst > 1 ? (size_t)smem : 0, s>>>(a, F, T);
  return cudaGetLastError();
}

}  // namespace fftgb
