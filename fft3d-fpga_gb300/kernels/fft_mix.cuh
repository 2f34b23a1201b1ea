// fft_mix.cuh - mixed-radix axis FFT for lengths 2^a 3^b 5^c (fft_mix.cu).
#pragma once

#include <cuda_runtime.h>

namespace fftgb {

constexpr int MIX_MAXN = 8192;   // longest axis
constexpr int MIX_MAXST = 16;    // most stages (3^8 = 6561 takes 8)

// Lines of n points along one axis of data [outer][n][inner]:
// nlines = outer * inner, point m of line (o, i) at (o*n + m)*inner + i.
struct MixArgs {
  const float2 *in = nullptr;
  float2 *out = nullptr;
  long long nlines = 0;
  long long inner = 1;
  int n = 0;              // axis length, 2 <= n <= MIX_MAXN
  int nst = 0;            // stages
  int rad[MIX_MAXST] = {};  // stage radices, first stage first (mix_radices)
  const float2 *w = nullptr;   // W_n^i = e^(-2 pi i i / n), i < n (FP64-generated)
  const float2 *wn = nullptr;  // real-data forms: W_2n^k, k = 0..n
  float scale = 1.0f;
  // four-step passes of long 1D transforms N = n1 * n2 (x[j1 + n1 j2]):
  // epi = 1, the column pass (lines j1 along j2, inner = n1): output k2 of
  // line j1 times W_N^(j1 k2) (conjugate for the inverse), from the two-level
  // table W_N^e = tw_hi[e >> 12] * tw_lo[e & 4095]; epi = 2, the row pass
  // (contiguous lines k2 of n1 points): output k1 of row k2 of transform o
  // stored at o*N + k2 + ep_n2*k1 (ep_n2 = n2, ep_N = N)
  int epi = 0;
  const float2 *tw_lo = nullptr;
  const float2 *tw_hi = nullptr;
  long long ep_n2 = 0;
  long long ep_N = 0;
  // set by the launchers: stage s's radix as its position in 16, 15, 12, 10,
  // 9, 8, 6, 5, 4, 3, 2, in bits 4s..4s+3 (the kernel reads no array of the
  // arguments by a runtime index, which would copy them to local memory)
  unsigned long long rcode = 0;
};

cudaError_t mix_kernels_init();
// Stage radices of n (first stage first); returns the stage count, or 0 when
// n is not 2^a 3^b 5^c, is 1, or is longer than MIX_MAXN.  simple: radix 16,
// 8, 4, 2, 5 and 3 stages only (no composite radices).
int mix_radices(int n, int *rad, bool simple = false);
// lines_per_cta: 0 picks the built-in choice.
cudaError_t launch_mix(int inverse, const MixArgs &a, cudaStream_t s,
                       int lines_per_cta = 0);
// The x pass of real-data transforms of rows of 2n reals (inner = 1).
// c2r = 0: in = the real rows read as n complex points, out = rows of n + 1
// spectrum values (the transform of the packed rows, then the split with
// W_2n^k through shared memory).  c2r = 1: in = rows of n + 1 spectrum values,
// combined on the load into the packed spectrum, out = the real rows
// (unnormalised inverse).
cudaError_t launch_mix_real(int c2r, const MixArgs &a, cudaStream_t s);

}  // namespace fftgb
