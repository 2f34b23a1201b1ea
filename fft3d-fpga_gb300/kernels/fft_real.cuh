// fft_real.cuh - contiguous-axis pass of real-data transforms (fft_real.cu).
#pragma once

#include <cuda_runtime.h>

namespace fftgb {

// Rows of N = 2M reals <-> M + 1 complex values.
struct RealArgs {
  const float2 *in;   // R2C: real rows read as M complex; C2R: M + 1 complex per row
  float2 *out;        // R2C: M + 1 complex per row; C2R: real rows written as M complex
  long long nrows;
  const float2 *tw;   // stage table of the M-point Stockham transform
  const float2 *wn;   // W_N^k, k = 0..M (FP64-generated)
  float scale;
};

cudaError_t real_kernels_init();
// log_m = log2(M) in 1..12 (N = 4 .. 8192)
cudaError_t launch_r2c_rows(int log_m, const RealArgs &a, cudaStream_t s);
cudaError_t launch_c2r_rows(int log_m, const RealArgs &a, cudaStream_t s);

}  // namespace fftgb
