// fft3d_cluster.cuh - single-launch 3D FFT of grids up to 2 MiB held in the
// distributed shared memory of one 16-CTA thread-block cluster.
#pragma once

#include <cuda_runtime.h>

namespace fftgb {

// Grids [batch][nz][ny][nx], complex64, x fastest; one cluster per grid.
struct C3dArgs {
  const float2 *in;
  float2 *out;
  long long batch;
  const float2 *tw_x;  // W_nx^m, m < nx
  const float2 *tw_y;  // W_ny^m
  const float2 *tw_z;  // W_nz^m
  float scale;
  int swap_io;         // 1: inverse (real/imaginary swap on load and store)
};

cudaError_t cluster3d_init();
// true when a kernel exists for the shape: every side 16, 32 or 64, so the
// grid (at most 2^18 points) fits one cluster's shared memory
bool cluster3d_available(int nx, int ny, int nz);
cudaError_t launch_cluster3d(int nx, int ny, int nz, const C3dArgs &a, cudaStream_t s);

}  // namespace fftgb
