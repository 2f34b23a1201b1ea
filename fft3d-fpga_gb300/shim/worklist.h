// worklist.h - host side of the persistent work-list kernel
// (kernels/fft_ragged.cu): units (grids or transforms) with up to three
// row/column passes each, turned into one item list and run by one launch.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "fftfpga_ext.h"

#include "../kernels/fft_ragged.cuh"

namespace fftgb {

constexpr int RG_MAX_PASSES = 3;

struct RgPass {
  int kind;         // RgItem::kind
  int log_l;        // transform length 2^log_l
  long long count;  // rows or columns of the pass
  long long inner;  // column stride (kinds 1, 2); ny (kind 3); nx (kind 4)
  int aux = 0;      // kind 3: rows per tile NJ; kind 4: radix R
};

struct RgUnit {
  long long base;    // first point
  long long points;  // points of the unit (chunking)
  int npasses;
  RgPass pass[RG_MAX_PASSES];
};

struct RgExec {
  RgItem *d_items = nullptr;
  int nitems = 0;
  int *d_counters = nullptr;  // [0] claim counter, then per (unit, pass)
  int ncounters = 0;
  int *d_status = nullptr;
};

// Item list for `units`: consecutive units form chunks of at most
// `chunk_points` points (at least one unit); pass p of chunk c is emitted at
// step c + p.  The last pass of every unit applies RgArgs::scale when
// `scale_last`.  False if a pass is not supported by the kernel.
bool rg_build(const std::vector<RgUnit> &units, long long chunk_points,
              bool scale_last, std::vector<RgItem> &items, int *ncounters);
int rg_tiles(const RgPass &p);
// FFTGB_* status codes
int rg_exec_create(const std::vector<RgItem> &items, int ncounters, RgExec *x);
void rg_exec_destroy(RgExec *x);
// zeroes the counters and launches the kernel on `s` (graph-capturable)
int rg_exec_launch(const RgExec &x, const float2 *in, float2 *out, int inv,
                   float scale, cudaStream_t s);
// FFTGB_ETIMEOUT (and clears the flag) if a dependency wait gave up
int rg_exec_status(const RgExec &x);
// chunk size in points: FFTGB_L2_CHUNK_MB (default 16 MiB of complex64)
long long rg_chunk_points();
// The two passes of a 3D grid as fused tiles (kinds 3 and 4, or 3 and z
// columns) when its shape fits them; sets u->pass / u->npasses (base and
// points are the caller's).  False otherwise (u->npasses then undefined).
bool rg_two_pass_unit(const fftgb_shape3 s, RgUnit *u);

}  // namespace fftgb
