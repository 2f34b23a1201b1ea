// spectral.cuh - element-wise kernels around the transforms: a spectral
// filter for plans whose last pass cannot apply it itself, and the fused
// residual / sum of squares of a least-squares loss.
#pragma once

#include <cuda_runtime.h>

namespace fftgb {

// d[i] *= G(kx, ky, kz) for the `batch` grids [nz][ny][nx] (any sides; a
// batch of sides that are not all powers of two below 2^32 points)
cudaError_t launch_filter(float2 *d, long long points, int nx, int ny, int nz, int kind,
                          cudaStream_t s);
// r = a - b (r may be NULL: not stored) and *sum += sum |a - b|^2 (FP64
// accumulation across blocks; the caller zeroes *sum first)
cudaError_t launch_sq_residual(const float2 *a, const float2 *b, float2 *r, long long n,
                               double *sum, cudaStream_t s);

}  // namespace fftgb
