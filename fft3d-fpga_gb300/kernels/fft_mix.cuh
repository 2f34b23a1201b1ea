// fft_mix.cuh - mixed-radix axis FFT for lengths 2^a 3^b 5^c (fft_mix.cu).
#pragma once

#include <cuda_runtime.h>

namespace fftgb {

constexpr int MIX_MAXN = 8192;   // longest axis
constexpr int MIX_MAXST = 16;    // most stages (3^8 = 6561 takes 8)

// Lines of n points along one axis of data [outer][n][inner]:
// nlines = outer * inner, point m of line (o, i) at (o*n + m)*inner + i.
struct MixArgs {
  const float2 *in;
  float2 *out;
  long long nlines;
  long long inner;
  int n;                  // axis length, 2 <= n <= MIX_MAXN
  int nst;                // stages
  int rad[MIX_MAXST];     // stage radices (2, 3, 4, 5, 8 or 16), first stage first
  const float2 *w;        // W_n^i = e^(-2 pi i i / n), i < n (FP64-generated)
  float scale;
};

cudaError_t mix_kernels_init();
// Stage radices of n (first stage first); returns the stage count, or 0 when
// n is not 2^a 3^b 5^c, is 1, or is longer than MIX_MAXN.
int mix_radices(int n, int *rad);
// lines_per_cta: 0 picks the built-in choice.
cudaError_t launch_mix(int inverse, const MixArgs &a, cudaStream_t s,
                       int lines_per_cta = 0);

}  // namespace fftgb
