// fft1d_cluster.cuh - single-pass cluster 1D FFT (N = L1*L2 points).
#pragma once

#include <cuda_runtime.h>

namespace fftgb {

struct C1dArgs {
  const float2 *in;
  float2 *out;
  long long count;      // transforms
  const float2 *tw_a;   // W_L2^m (over n2)
  const float2 *tw_b;   // W_L1^m (over n1)
  const float2 *tw4_lo; // W_N^e = lo[e & mask] * hi[e >> bits]
  const float2 *tw4_hi;
  int tw4_bits;
  int bitrev;           // 1: fftfpgaf_c2c_1d output order
  float scale;
  int swap_io;
  int push;             // 0: remote loads (k_1d_cluster); 1: bulk copies (k_1d_push)
};

cudaError_t cluster1d_init();
// true when a cluster kernel of c CTAs (0: the default size) exists for n;
// returns its L1, L2
bool cluster1d_available(int n, int c, int *l1, int *l2);
// the cluster sizes instantiated for n (default first); returns the count
int cluster1d_sizes(int n, int *sizes, int max_sizes);
cudaError_t launch_cluster1d(int n, int c, const C1dArgs &a, cudaStream_t s);
// forms instantiated for (n, c): bit 0 remote loads, bit 1 bulk copies;
// bit 2 set when bulk copies are the measured default (0: no kernel)
int cluster1d_exchange_forms(int n, int c);
// 1 if a bounded wait of the bulk-copy form gave up since the last call
// (synchronises; clears the flag), 0 if not, -1 on a CUDA error
int cluster1d_status_and_clear();
cudaError_t cluster1d_expire_wait(unsigned polls);

}  // namespace fftgb
