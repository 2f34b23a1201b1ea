// fft_ragged.cuh - persistent work-list kernel (fft_ragged.cu): ragged
// batches of 3D grids in one launch.
#pragma once

#include <cuda_runtime.h>

namespace fftgb {

// One tile of one pass of one unit (a grid or a transform).
struct RgItem {
  long long base;   // first point of the unit
  long long first;  // first row (kind 0) or column (kind 1) of the tile
  long long count;  // rows or columns of this pass of this unit
  long long inner;  // column stride (kind 1)
  int kind;         // 0: rows (contiguous axis), 1: strided columns, in place,
                    // 3: 3D pass A: x FFT (L = nx) and the aux-point y FFT
                    //    over rows y = R*j + r of 8192/(L*aux) planes, twiddle
                    //    W_ny^(r*k1), rows r*aux + k1 stored (inner = ny,
                    //    count = nz; tile first = plane_group*R + r),
                    // 4: 3D pass B: radix-aux over the residue rows r*nj + k1
                    //    and the z FFT (L = nz) of X = 8192/(aux*L) columns,
                    //    in place (inner = nx, count = nj * nx / X; tile first
                    //    = k1 * (nx / X) + x block)
  int aux;          // kind 3: rows per pass-A tile (NJ); kind 4: radix R
  int scale;        // 1: multiply the outputs by RgArgs::scale (last pass)
  int log_l;        // axis length 2^log_l
  int src_in;       // 1: read the batch input, 0: work in place in the output
  int dep;          // counter to wait for (-1: none)
  int dep_target;   // ... until it reaches this value
  int done_id;      // counter this tile increments when finished
};

struct RgArgs {
  const float2 *in;
  float2 *out;
  const RgItem *items;
  int nitems;
  int *counter;  // next item to claim (zeroed before each launch)
  int *done;     // per (grid, axis) finished-tile counters (zeroed)
  int *status;   // set to 1 if a bounded wait gave up
  const float2 *tw[13];  // stage tables of the per-axis plans, by log2 L
  const float2 *tw16[13];  // stage tables of Stock<L, 16> (kinds 3, 4)
  const float2 *tww[13];   // W_L^m, m < L (kind 3's y twiddle)
  float scale;
};

bool ragged_axis_supported(int log_l);
// kinds 3 (log_l = log2 nx, aux = NJ) and 4 (log_l = log2 nz, aux = R)
bool ragged_fused_supported(int kind, int log_l, int aux);
int ragged_fused_tile_points();  // points per kind-3/4 tile
int ragged_rows_per_tile(int log_l);
int ragged_cols_per_tile(int log_l);
cudaError_t ragged_init(int device);
cudaError_t launch_ragged(const RgArgs &a, int inverse, cudaStream_t s);
// Runs the dependency wait's give-up path once (a wait on *ctr reaching
// INT_MAX that gives up after `polls` polls and sets *status); synchronises.
cudaError_t ragged_expire_wait(const int *ctr, int *status, unsigned polls);

}  // namespace fftgb
