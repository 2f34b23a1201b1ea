// ragged.cu - ragged batches of 3D grids with independent power-of-two
// shapes (no counterpart in the reference, whose bitstreams fix one N per
// build, kernels/common/fft_config.h.in:6-15).
//
// The batch is executed as one CUDA graph: every grid's axis passes are
// recorded once per (input, output, direction, stream) and replayed with a
// single cudaGraphLaunch.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "fftfpga_ext.h"

struct fftgb_ragged_s {
  std::vector<fftgb_shape3> shapes;
  std::vector<size_t> offset;  // first point of each grid
  std::vector<fftgb_plan> plans;
  size_t points;
  unsigned flags;
  // cached graph
  cudaGraphExec_t exec;
  const void *g_in;
  void *g_out;
  int g_inv;
  cudaStream_t g_stream;
};

static bool pow2u(unsigned v) { return v && !(v & (v - 1)); }

extern "C" int fftgb_ragged_plan(fftgb_ragged *plan, const fftgb_shape3 *shapes,
                                 unsigned count, unsigned flags) {
  if (plan == NULL || shapes == NULL || count == 0) return FFTGB_EINVAL;
  *plan = NULL;
  fftgb_ragged r = new fftgb_ragged_s();
  r->points = 0;
  r->flags = flags;
  r->exec = NULL;
  r->g_in = NULL;
  r->g_out = NULL;
  r->g_inv = -1;
  r->g_stream = NULL;
  for (unsigned i = 0; i < count; i++) {
    const fftgb_shape3 s = shapes[i];
    if (!pow2u(s.nx) || !pow2u(s.ny) || !pow2u(s.nz)) {
      fftgb_ragged_destroy(r);
      return FFTGB_EINVAL;
    }
    fftgb_plan p = NULL;
    int rc = fftgb_plan_3d(&p, s.nx, s.ny, s.nz, 1, flags);
    if (rc) {
      fftgb_ragged_destroy(r);
      return rc;
    }
    r->shapes.push_back(s);
    r->offset.push_back(r->points);
    r->plans.push_back(p);
    r->points += (size_t)s.nx * s.ny * s.nz;
  }
  *plan = r;
  return FFTGB_OK;
}

extern "C" void fftgb_ragged_destroy(fftgb_ragged r) {
  if (!r) return;
  if (r->exec) cudaGraphExecDestroy(r->exec);
  for (fftgb_plan p : r->plans) fftgb_plan_destroy(p);
  delete r;
}

extern "C" size_t fftgb_ragged_points(fftgb_ragged r) {
  return r ? r->points : 0;
}

extern "C" int fftgb_ragged_exec(fftgb_ragged r, const void *d_in, void *d_out,
                                 int inverse, void *stream) {
  if (!r || !d_in || !d_out || d_in == d_out) return FFTGB_EINVAL;
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
    int rc = FFTGB_OK;
    for (size_t i = 0; i < r->plans.size() && rc == FFTGB_OK; i++) {
      const float2 *src = (const float2 *)d_in + r->offset[i];
      float2 *dst = (float2 *)d_out + r->offset[i];
      rc = fftgb_exec(r->plans[i], src, dst, inv, 1.0f, cap);
    }
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
