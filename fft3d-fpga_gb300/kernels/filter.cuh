// filter.cuh - spectral filters that a transform can apply to its outputs
// in the same pass that stores them (no extra pass over HBM).
#pragma once

#include <cuda_runtime.h>

namespace fftgb {

// Filter kinds (fftfpga_ext.h: FFTGB_FILTER_*).
constexpr int FILTER_NONE = 0;
// Poisson Green's function G(k) = 1/|k|^2, G(0) = 0, on the integer
// wavenumber grid k = n * fftfreq(n) per axis (index i < (n + 1)/2 is i, the
// rest i - n: for even n the index n/2 is -n/2, for odd n the middle index
// (n - 1)/2 stays positive).  |k|^2 is an exact integer in FP32 for sides up
// to 4096 (and within one rounding above), and the division is IEEE-rounded,
// so G is the correctly rounded 1/|k|^2.
constexpr int FILTER_POISSON = 1;

__device__ __forceinline__ int fftfreq_k(int i, int n) { return i < (n + 1) / 2 ? i : i - n; }

// Real factor of the output at wavenumber index (kx, ky, kz).
__device__ __forceinline__ float filter_g(int kind, int kx, int ky, int kz, int nx, int ny,
                                          int nz) {
  if (kind != FILTER_POISSON) return 1.0f;
  const int fx = fftfreq_k(kx, nx), fy = fftfreq_k(ky, ny), fz = fftfreq_k(kz, nz);
  const float k2 = (float)(fx * fx + fy * fy + fz * fz);
  return k2 > 0.0f ? 1.0f / k2 : 0.0f;
}

}  // namespace fftgb
