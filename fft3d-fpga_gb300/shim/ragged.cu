// ragged.cu - ragged batches of 3D grids with independent power-of-two
// shapes (no counterpart in the reference, whose bitstreams fix one N per
// build, kernels/common/fft_config.h.in:6-15).
//
// Persistent form (every axis length 16..512): the whole batch is one work
// list executed by one persistent kernel launch (kernels/fft_ragged.cu),
// recorded with the zeroing of its counters into a CUDA graph.
// Graph-of-plans form (other shapes, or FFTGB_RAGGED_GRAPH=1): each grid's
// own plan (with its tuned variant) is recorded into one CUDA graph.
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "fftfpga_ext.h"
#include "../kernels/fft_ragged.cuh"

namespace fftgb {
int internal_ensure_device(int *device);
const float2 *internal_axis_tw(int log_l);
void internal_set_err(const char *msg);
}  // namespace fftgb

using namespace fftgb;

struct fftgb_ragged_s {
  std::vector<fftgb_shape3> shapes;
  std::vector<size_t> offset;  // first point of each grid
  size_t points;
  unsigned flags;
  bool persistent;
  // persistent form
  RgItem *d_items;
  int nitems;
  int *d_counters;  // [0] claim counter, [1..] per (grid, axis) done counters
  int ncounters;
  int *d_status;
  // graph-of-plans form
  std::vector<fftgb_plan> plans;
  // cached graph
  cudaGraphExec_t exec;
  const void *g_in;
  void *g_out;
  int g_inv;
  cudaStream_t g_stream;
};

static bool pow2u(unsigned v) { return v && !(v & (v - 1)); }
static int log2u(unsigned v) {
  int r = 0;
  while ((1u << r) < v) r++;
  return r;
}

static bool build_items(fftgb_ragged r, std::vector<RgItem> &items) {
  // per grid, the present axes in execution order (x, y, z)
  struct Ax {
    int kind, log_l;
    long long count, inner, per_tile;
  };
  std::vector<std::vector<Ax>> axes(r->shapes.size());
  for (size_t g = 0; g < r->shapes.size(); g++) {
    const fftgb_shape3 s = r->shapes[g];
    if (s.nx > 1) {
      if (!ragged_axis_supported(log2u(s.nx))) return false;
      axes[g].push_back({0, log2u(s.nx), (long long)s.ny * s.nz, 1,
                         ragged_rows_per_tile(log2u(s.nx))});
    }
    if (s.ny > 1) {
      if (!ragged_axis_supported(log2u(s.ny))) return false;
      axes[g].push_back({1, log2u(s.ny), (long long)s.nx * s.nz, (long long)s.nx,
                         ragged_cols_per_tile(log2u(s.ny))});
    }
    if (s.nz > 1) {
      if (!ragged_axis_supported(log2u(s.nz))) return false;
      axes[g].push_back({1, log2u(s.nz), (long long)s.nx * s.ny,
                         (long long)s.nx * s.ny, ragged_cols_per_tile(log2u(s.nz))});
    }
    if (axes[g].empty()) return false;
  }
  for (int phase = 0; phase < 3; phase++) {
    for (size_t g = 0; g < r->shapes.size(); g++) {
      if ((int)axes[g].size() <= phase) continue;
      const Ax &a = axes[g][(size_t)phase];
      const long long tiles = (a.count + a.per_tile - 1) / a.per_tile;
      int dep = -1, target = 0;
      if (phase > 0) {
        const Ax &p = axes[g][(size_t)phase - 1];
        dep = 1 + (int)g * 3 + phase - 1;
        target = (int)((p.count + p.per_tile - 1) / p.per_tile);
      }
      for (long long t = 0; t < tiles; t++) {
        RgItem it;
        it.base = (long long)r->offset[g];
        it.first = t * a.per_tile;
        it.count = a.count;
        it.inner = a.inner;
        it.kind = a.kind;
        it.log_l = a.log_l;
        it.src_in = phase == 0 ? 1 : 0;
        it.dep = dep;
        it.dep_target = target;
        it.done_id = 1 + (int)g * 3 + phase;
        items.push_back(it);
      }
    }
  }
  return true;
}

extern "C" int fftgb_ragged_plan(fftgb_ragged *plan, const fftgb_shape3 *shapes,
                                 unsigned count, unsigned flags) {
  if (plan == NULL || shapes == NULL || count == 0) return FFTGB_EINVAL;
  *plan = NULL;
  int device = 0;
  int rc = internal_ensure_device(&device);
  if (rc) return rc;
  fftgb_ragged r = new fftgb_ragged_s();
  r->points = 0;
  r->flags = flags;
  r->persistent = false;
  r->d_items = NULL;
  r->nitems = 0;
  r->d_counters = NULL;
  r->ncounters = 0;
  r->d_status = NULL;
  r->exec = NULL;
  r->g_in = NULL;
  r->g_out = NULL;
  r->g_inv = -1;
  r->g_stream = NULL;
  for (unsigned i = 0; i < count; i++) {
    const fftgb_shape3 s = shapes[i];
    if (!pow2u(s.nx) || !pow2u(s.ny) || !pow2u(s.nz)) {
      fftgb_ragged_destroy(r);
      internal_set_err("ragged shapes must be powers of two");
      return FFTGB_EINVAL;
    }
    r->shapes.push_back(s);
    r->offset.push_back(r->points);
    r->points += (size_t)s.nx * s.ny * s.nz;
  }
  std::vector<RgItem> items;
  const char *force_graph = getenv("FFTGB_RAGGED_GRAPH");
  const bool want_persistent =
      (flags & FFTGB_PREC_MASK) == FFTGB_PREC_FP32 &&
      !(force_graph && *force_graph == '1');
  if (want_persistent && build_items(r, items) && ragged_init(device) == cudaSuccess) {
    r->nitems = (int)items.size();
    r->ncounters = 1 + 3 * (int)count;
    if (cudaMalloc((void **)&r->d_items, items.size() * sizeof(RgItem)) != cudaSuccess ||
        cudaMalloc((void **)&r->d_counters, r->ncounters * sizeof(int)) != cudaSuccess ||
        cudaMalloc((void **)&r->d_status, sizeof(int)) != cudaSuccess) {
      cudaGetLastError();
      fftgb_ragged_destroy(r);
      internal_set_err("ragged plan allocation failed");
      return FFTGB_ENOMEM;
    }
    cudaMemcpy(r->d_items, items.data(), items.size() * sizeof(RgItem),
               cudaMemcpyHostToDevice);
    cudaMemset(r->d_status, 0, sizeof(int));
    r->persistent = true;
  } else {
    for (unsigned i = 0; i < count; i++) {
      fftgb_plan p = NULL;
      rc = fftgb_plan_3d(&p, shapes[i].nx, shapes[i].ny, shapes[i].nz, 1, flags);
      if (rc) {
        fftgb_ragged_destroy(r);
        return rc;
      }
      r->plans.push_back(p);
    }
  }
  *plan = r;
  return FFTGB_OK;
}

extern "C" void fftgb_ragged_destroy(fftgb_ragged r) {
  if (!r) return;
  if (r->exec) cudaGraphExecDestroy(r->exec);
  for (fftgb_plan p : r->plans) fftgb_plan_destroy(p);
  if (r->d_items) cudaFree(r->d_items);
  if (r->d_counters) cudaFree(r->d_counters);
  if (r->d_status) cudaFree(r->d_status);
  delete r;
}

extern "C" size_t fftgb_ragged_points(fftgb_ragged r) {
  return r ? r->points : 0;
}

extern "C" int fftgb_ragged_launches(fftgb_ragged r) {
  if (!r) return 0;
  if (r->persistent) return 1;
  int n = 0;
  for (fftgb_plan p : r->plans) n += fftgb_plan_launches(p);
  return n;
}

extern "C" int fftgb_ragged_status(fftgb_ragged r) {
  if (!r || !r->persistent) return FFTGB_OK;
  int st = 0;
  if (cudaMemcpy(&st, r->d_status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return FFTGB_ECUDA;
  if (st) {
    cudaMemset(r->d_status, 0, sizeof(int));
    internal_set_err("a ragged-batch dependency wait gave up");
    return FFTGB_ETIMEOUT;
  }
  return FFTGB_OK;
}

static int record(fftgb_ragged r, const void *d_in, void *d_out, int inv,
                  cudaStream_t cap) {
  if (r->persistent) {
    if (cudaMemsetAsync(r->d_counters, 0, r->ncounters * sizeof(int), cap) !=
        cudaSuccess)
      return FFTGB_ECUDA;
    RgArgs a;
    a.in = (const float2 *)d_in;
    a.out = (float2 *)d_out;
    a.items = r->d_items;
    a.nitems = r->nitems;
    a.counter = r->d_counters;
    a.done = r->d_counters;
    a.status = r->d_status;
    for (int l = 0; l < 13; l++) a.tw[l] = (l >= 1) ? internal_axis_tw(l) : NULL;
    return launch_ragged(a, inv, cap) == cudaSuccess ? FFTGB_OK : FFTGB_ECUDA;
  }
  int rc = FFTGB_OK;
  for (size_t i = 0; i < r->plans.size() && rc == FFTGB_OK; i++) {
    const float2 *src = (const float2 *)d_in + r->offset[i];
    float2 *dst = (float2 *)d_out + r->offset[i];
    rc = fftgb_exec(r->plans[i], src, dst, inv, 1.0f, cap);
  }
  return rc;
}

extern "C" int fftgb_ragged_exec(fftgb_ragged r, const void *d_in, void *d_out,
                                 int inverse, void *stream) {
  if (!r || !d_in || !d_out) return FFTGB_EINVAL;
  const size_t bytes = r->points * 8;
  const char *a = (const char *)d_in, *b = (const char *)d_out;
  if (a < b + bytes && b < a + bytes) {
    internal_set_err("ragged input and output overlap");
    return FFTGB_EINVAL;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int inv = inverse ? 1 : 0;
  if (!(r->exec && r->g_in == d_in && r->g_out == d_out && r->g_inv == inv &&
        r->g_stream == s)) {
    if (r->exec) {
      cudaGraphExecDestroy(r->exec);
      r->exec = NULL;
    }
    // capture on a private stream so the caller's stream may be the legacy
    // default stream
    cudaStream_t cap;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess)
      return FFTGB_ECUDA;
    cudaGraph_t graph;
    if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) !=
        cudaSuccess) {
      cudaStreamDestroy(cap);
      return FFTGB_ECUDA;
    }
    const int rc = record(r, d_in, d_out, inv, cap);
    cudaError_t e = cudaStreamEndCapture(cap, &graph);
    cudaStreamDestroy(cap);
    if (rc != FFTGB_OK) {
      if (e == cudaSuccess) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) return FFTGB_ECUDA;
    e = cudaGraphInstantiate(&r->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      r->exec = NULL;
      return FFTGB_ECUDA;
    }
    r->g_in = d_in;
    r->g_out = d_out;
    r->g_inv = inv;
    r->g_stream = s;
  }
  if (cudaGraphLaunch(r->exec, s) != cudaSuccess) return FFTGB_ECUDA;
  return FFTGB_OK;
}
