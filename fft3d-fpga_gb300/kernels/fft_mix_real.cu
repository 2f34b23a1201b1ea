// fft_mix_real.cu - the real-data instantiations of the mixed-radix axis
// kernel (kernels/fft_mix_impl.cuh): the x pass of R2C / C2R transforms
// whose rows of 2n reals are packed as n complex points, with the split into
// (R2C) or the combination from (C2R) the n + 1 spectrum values fused into
// the transform.  A translation unit of its own so that it compiles beside
// fft_mix.cu.
#include "fft_mix_impl.cuh"

namespace fftgb {

namespace {
MixFn g_mix_real[2][2];  // [c2r][more than 256 threads]
MixPairRealTable g_mix2_real = {};  // two-stage forms
MixTripleRealTable g_mix3_real = {};  // three-stage forms
constexpr int MIX_REAL_SMEM_MAX = 100 * 1024;
bool g_mix_real_ready = false;

bool getenv_generic() {  // FFTGB_MIX_GENERIC=1: the kernel that holds every radix
  const char *e = getenv("FFTGB_MIX_GENERIC");
  return e && atoi(e) == 1;
}
}  // namespace

cudaError_t mix_real_init() {
  if (g_mix_real_ready) return cudaSuccess;
  g_mix_real[0][0] = k_mix<false, false, 256, 1>;
  g_mix_real[0][1] = k_mix<false, false, MIX_THREADS, 1>;
  g_mix_real[1][0] = k_mix<true, false, 256, 2>;
  g_mix_real[1][1] = k_mix<true, false, MIX_THREADS, 2>;
  for (int d = 0; d < 2; d++)
    for (int big = 0; big < 2; big++) {
      const cudaError_t e = cudaFuncSetAttribute((const void *)g_mix_real[d][big],
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 MIX_REAL_SMEM_MAX);
      if (e != cudaSuccess) return e;
    }
  mix2_fill_real_a(g_mix2_real);
  mix2_fill_real_b(g_mix2_real);
  mix2_fill_real_c(g_mix2_real);
  for (int r0 = 0; r0 < 11; r0++)
    for (int r1 = 0; r1 < 11; r1++)
      for (int d = 0; d < 2; d++) {
        MixFn f = g_mix2_real[r0][r1][d];
        if (!f) continue;
        const cudaError_t e = cudaFuncSetAttribute(
            (const void *)f, cudaFuncAttributeMaxDynamicSharedMemorySize, MIX_REAL_SMEM_MAX);
        if (e != cudaSuccess) return e;
      }
  mix3_fill_real_d(g_mix3_real);
  mix3_fill_real_e(g_mix3_real);
  mix3_fill_real_f(g_mix3_real);
  mix3_fill_real_g(g_mix3_real);
  mix3_fill_real_h(g_mix3_real);
  mix3_fill_real_i(g_mix3_real);
  for (int r0 = 0; r0 < 11; r0++)
    for (int r1 = 0; r1 < 11; r1++)
      for (int r2 = 0; r2 < 11; r2++)
        for (int d = 0; d < 2; d++) {
          MixFn f = g_mix3_real[r0][r1][r2][d];
          if (!f) continue;
          const cudaError_t e = cudaFuncSetAttribute(
              (const void *)f, cudaFuncAttributeMaxDynamicSharedMemorySize, MIX_REAL_SMEM_MAX);
          if (e != cudaSuccess) return e;
        }
  g_mix_real_ready = true;
  return cudaSuccess;
}

cudaError_t launch_mix_real(int c2r, const MixArgs &a, cudaStream_t s) {
  if (!g_mix_real_ready || !a.wn) return cudaErrorInvalidValue;
  MixShape sh;
  const cudaError_t e = mix_shape(a, 0, true, &sh);
  if (e != cudaSuccess) return e;
  MixArgs b = a;
  b.rcode = sh.rcode;
  MixFn f = g_mix_real[c2r ? 1 : 0][sh.big ? 1 : 0];
  if (!sh.big && !getenv_generic()) {
    MixFn fs = nullptr;
    if (a.nst == 2) fs = g_mix2_real[mix_rank(a.rad[0])][mix_rank(a.rad[1])][c2r ? 1 : 0];
    if (a.nst == 3)
      fs = g_mix3_real[mix_rank(a.rad[0])][mix_rank(a.rad[1])][mix_rank(a.rad[2])][c2r ? 1 : 0];
    if (fs) f = fs;
  }
  f<<<(unsigned)sh.grid, sh.F * sh.T, sh.smem, s>>>(b, sh.F, sh.T);
  return cudaGetLastError();
}

}  // namespace fftgb
