// fft_ragged.cuh - persistent ragged-batch kernel (fft_ragged.cu).
#pragma once

#include <cuda_runtime.h>

namespace fftgb {

// One tile of one axis pass of one grid.
struct RgItem {
  long long base;   // first point of the grid
  long long first;  // first row (kind 0) or column (kind 1) of the tile
  long long count;  // rows or columns of this axis pass of this grid
  long long inner;  // column stride (kind 1)
  int kind;         // 0: rows (x axis), 1: strided columns (y, z axes)
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
};

bool ragged_axis_supported(int log_l);
int ragged_rows_per_tile(int log_l);
int ragged_cols_per_tile(int log_l);
cudaError_t ragged_init(int device);
cudaError_t launch_ragged(const RgArgs &a, int inverse, cudaStream_t s);

}  // namespace fftgb
