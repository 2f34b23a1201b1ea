// fft3d_fused.cuh - arguments and launchers of the two-pass 3D kernels.
#pragma once

#include <cuda_runtime.h>

namespace fftgb {

// Grids [batch][nz][ny][nx], complex64, x fastest.
struct FusedArgs {
  const float2 *in;
  float2 *out;
  int nx, ny, nz;
  long long batch;
  const float2 *tw_x;  // W_nx^m
  const float2 *tw_j;  // W_(ny/R)^m (pass A)
  const float2 *tw_y;  // W_ny^m (pass A, R > 1)
  const float2 *tw_z;  // W_nz^m (pass B)
  float scale;
  int swap_io;
  int twb = 0;  // 1: W_ny^(r*k1) is applied by pass B to its inputs (once
                // per tile per residue row), not by pass A to its outputs
  int filter = 0;  // pass B (k_rz, k_rz_tma): multiply each output by the
                   // spectral filter of this kind (filter.cuh) at its (kx, ky, kz)
};

cudaError_t fused_kernels_init();
// ept: points per thread of the one-tile kernels (16, or 8 where built)
bool fused_xy_available(int nx, int nj, int ept = 16);
bool fused_rz_available(int nz, int r, int x, int ept = 16);
// pass A over rows y = R*j + r with R = ny / nj
// pdl: programmatic dependent launch after the previous kernel of stream s
cudaError_t launch_fused_xy(int nj, const FusedArgs &a, cudaStream_t s, bool pdl = false,
                            int ept = 16);
// pass B with R = ny / nj residue rows and x-blocks of `x` columns
cudaError_t launch_fused_rz(int r, int x, const FusedArgs &a, cudaStream_t s,
                            bool pdl = false, int ept = 16);
// pass A as a persistent kernel whose tiles arrive by TMA tensor copies
// (fft3d_fused_tma.cu; nx <= 256); cudaErrorNotSupported when the driver
// has no tensor-map encoder, cudaErrorMisalignedAddress for an input that
// is not 16-byte aligned
cudaError_t fused_tma_init();
bool fused_xy_tma_available(int nx, int nj);
cudaError_t launch_fused_xy_tma(int nj, const FusedArgs &a, cudaStream_t s, bool pdl = false);
// pass B likewise (nz, r, x) = (256, 4, 8), (256, 8, 4) or (128, 2, 16);
// cudaErrorNotSupported for other shapes
bool fused_rz_tma_available(int nz, int r, int x);
cudaError_t launch_fused_rz_tma(int r, int x, const FusedArgs &a, cudaStream_t s,
                                bool pdl = false);
// Passes A and B of a group of up to FUSED_TMA_GRIDS same-shape grids at
// element offsets off[] from a.in / a.out (a ragged batch's grids of one
// shape; a.batch is ignored), one persistent launch each, tensor maps per
// grid.  cudaErrorMisalignedAddress when a grid is not 16-byte aligned.
constexpr int FUSED_TMA_GRIDS = 14;
cudaError_t launch_fused_xy_tma_grids(int nj, const FusedArgs &a, const long long *off,
                                      int ngrids, cudaStream_t s, bool pdl = false);
cudaError_t launch_fused_rz_tma_grids(int r, int x, const FusedArgs &a, const long long *off,
                                      int ngrids, cudaStream_t s, bool pdl = false);
// 1 if a TMA completion wait of pass A or B gave up since the last call
// (clears it), -1 on a CUDA error
int fused_tma_status_and_clear();
cudaError_t fused_tma_expire_wait(unsigned polls);

}  // namespace fftgb
