// fft_blue.cuh - any-length axis FFT by Bluestein's algorithm (fft_blue.cu).
#pragma once

#include <cuda_runtime.h>

namespace fftgb {

// Lines of n points along one axis of data [outer][n][inner]:
// nlines = outer * inner, point m of line (o, i) at (o*n + m)*inner + i.
struct BlueArgs {
  const float2 *in;
  float2 *out;
  long long nlines;
  long long inner;
  int n;              // axis length, 2 <= n, 2n - 1 <= M
  const float2 *tw;   // stage table of the M-point Stockham transform (Cfg<M>)
  const float2 *w;    // chirp e^(-i pi m^2 / n), m < n
  const float2 *H;    // DFT_M of the chirp filter, divided by M
  float scale;
};

cudaError_t blue_kernels_init();
int blue_length(int n);  // M: the power of two >= 2n - 1 (at least 4)
// log_m = log2(M) in 2..12 (n <= 2048)
cudaError_t launch_blue(int log_m, int inverse, const BlueArgs &a, cudaStream_t s);

}  // namespace fftgb
