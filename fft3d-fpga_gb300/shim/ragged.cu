// ragged.cu - ragged batches of 3D grids with independent power-of-two
// shapes (no counterpart in the reference, whose bitstreams fix one N per
// build, kernels/common/fft_config.h.in:6-15).
//
// Persistent form (every axis length 16..512): the whole batch is one work
// list executed by one persistent kernel launch (kernels/fft_ragged.cu),
// recorded with the zeroing of its counters into a CUDA graph.
// Grids of the shapes the uniform plans run fastest (nz = ny = 256, nx 128
// or 256: both passes TMA-fed) leave the work list: each such shape runs as
// grouped launches of the uniform plan's two passes over up to 14 grids at
// their own offsets (FFTGB_RAGGED_NO_GROUP=1 keeps every grid in the list).
// Graph-of-plans form (other shapes, or FFTGB_RAGGED_GRAPH=1): each grid's
// own plan (with its tuned variant) is recorded into one CUDA graph.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "fftfpga_ext.h"
#include "../kernels/fft3d_fused.cuh"
#include "../kernels/fft_ragged.cuh"
#include "worklist.h"

namespace fftgb {
int internal_ensure_device(int *device);
unsigned internal_device_generation();
const float2 *internal_axis_tw(int log_l);
const float2 *internal_stage_tw16(int log_l);
const float2 *internal_w_table(int log_l);
void internal_set_err(const char *msg);
}  // namespace fftgb

using namespace fftgb;

// ------------------------------------------------------------ work lists
namespace fftgb {

// rows / columns per tile (kinds 0-2); kinds 3, 4 number their tiles
static long long rg_per_tile(const RgPass &p) {
  if (p.kind >= 3) return 1;
  return p.kind == 0 ? ragged_rows_per_tile(p.log_l) : ragged_cols_per_tile(p.log_l);
}

int rg_tiles(const RgPass &p) {
  const long long pts = ragged_fused_tile_points();
  if (p.kind == 3) {  // (nz / P) plane groups x R residues
    const long long planes = pts / ((1LL << p.log_l) * p.aux);
    return (int)((p.count / planes) * (p.inner / p.aux));
  }
  if (p.kind == 4) return (int)p.count;  // nj * nx / X
  const long long per = rg_per_tile(p);
  return (int)((p.count + per - 1) / per);
}

bool rg_build(const std::vector<RgUnit> &units, long long chunk_points,
              bool scale_last, std::vector<RgItem> &items, int *ncounters) {
  items.clear();
  if (units.empty()) return false;
  for (const RgUnit &u : units) {
    if (u.npasses < 1 || u.npasses > RG_MAX_PASSES) return false;
    for (int p = 0; p < u.npasses; p++)
    {
      const RgPass &q = u.pass[p];
      if (q.kind >= 3 ? !ragged_fused_supported(q.kind, q.log_l, q.aux)
                      : (!ragged_axis_supported(q.log_l) || q.kind < 0 ||
                         q.kind == 2))
        return false;
    }
  }
  // chunks: runs of consecutive units of at most chunk_points (at least one)
  std::vector<size_t> first;  // first unit of each chunk
  long long acc = 0;
  for (size_t i = 0; i < units.size(); i++) {
    if (first.empty() || acc + units[i].points > chunk_points) {
      first.push_back(i);
      acc = 0;
    }
    acc += units[i].points;
  }
  first.push_back(units.size());
  const int nchunks = (int)first.size() - 1;
  // pass p of chunk c at step c + p: a pass's inputs were produced one step
  // earlier (still in L2 for small chunks) and every dependency precedes its
  // dependents in the list
  for (int step = 0; step < nchunks + RG_MAX_PASSES - 1; step++) {
    for (int p = 0; p < RG_MAX_PASSES; p++) {
      const int c = step - p;
      if (c < 0 || c >= nchunks) continue;
      for (size_t u = first[(size_t)c]; u < first[(size_t)c + 1]; u++) {
        const RgUnit &un = units[u];
        if (p >= un.npasses) continue;
        const RgPass &ps = un.pass[p];
        const int tiles = rg_tiles(ps);
        const long long per = rg_per_tile(ps);
        for (int t = 0; t < tiles; t++) {
          RgItem it;
          it.base = un.base;
          it.first = (long long)t * per;
          it.count = ps.count;
          it.inner = ps.inner;
          it.kind = ps.kind;
          it.aux = ps.aux;
          it.scale = scale_last && p == un.npasses - 1 ? 1 : 0;
          it.log_l = ps.log_l;
          it.src_in = p == 0 ? 1 : 0;
          it.dep = p > 0 ? 1 + (int)u * RG_MAX_PASSES + p - 1 : -1;
          it.dep_target = p > 0 ? rg_tiles(un.pass[p - 1]) : 0;
          it.done_id = 1 + (int)u * RG_MAX_PASSES + p;
          items.push_back(it);
        }
      }
    }
  }
  *ncounters = 1 + RG_MAX_PASSES * (int)units.size();
  return true;
}

int rg_exec_create(const std::vector<RgItem> &items, int ncounters, RgExec *x) {
  *x = RgExec();
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || ragged_init(device) != cudaSuccess)
    return FFTGB_ECUDA;
  x->nitems = (int)items.size();
  x->ncounters = ncounters;
  if (cudaMalloc((void **)&x->d_items, items.size() * sizeof(RgItem)) != cudaSuccess ||
      cudaMalloc((void **)&x->d_counters, (size_t)ncounters * sizeof(int)) != cudaSuccess ||
      cudaMalloc((void **)&x->d_status, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    rg_exec_destroy(x);
    return FFTGB_ENOMEM;
  }
  if (cudaMemcpy(x->d_items, items.data(), items.size() * sizeof(RgItem),
                 cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(x->d_status, 0, sizeof(int)) != cudaSuccess) {
    rg_exec_destroy(x);
    return FFTGB_ECUDA;
  }
  return FFTGB_OK;
}

void rg_exec_destroy(RgExec *x) {
  if (x->d_items) cudaFree(x->d_items);
  if (x->d_counters) cudaFree(x->d_counters);
  if (x->d_status) cudaFree(x->d_status);
  *x = RgExec();
}

int rg_exec_launch(const RgExec &x, const float2 *in, float2 *out, int inv,
                   float scale, cudaStream_t s) {
  if (cudaMemsetAsync(x.d_counters, 0, (size_t)x.ncounters * sizeof(int), s) !=
      cudaSuccess)
    return FFTGB_ECUDA;
  RgArgs a;
  a.in = in;
  a.out = out;
  a.items = x.d_items;
  a.nitems = x.nitems;
  a.counter = x.d_counters;
  a.done = x.d_counters;
  a.status = x.d_status;
  for (int l = 0; l < 13; l++) {
    a.tw[l] = (l >= 1) ? internal_axis_tw(l) : NULL;
    a.tw16[l] = (l >= 1) ? internal_stage_tw16(l) : NULL;
    a.tww[l] = (l >= 1) ? internal_w_table(l) : NULL;
  }
  a.scale = scale;
  return launch_ragged(a, inv, s) == cudaSuccess ? FFTGB_OK : FFTGB_ECUDA;
}

int rg_exec_status(const RgExec &x) {
  int st = 0;
  if (cudaMemcpy(&st, x.d_status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return FFTGB_ECUDA;
  if (st) {
    cudaMemset(x.d_status, 0, sizeof(int));
    internal_set_err("a persistent work-list dependency wait gave up");
    return FFTGB_ETIMEOUT;
  }
  return FFTGB_OK;
}

long long rg_chunk_points() {
  const char *e = getenv("FFTGB_L2_CHUNK_MB");
  long long mb = e && *e ? atoll(e) : 16;
  if (mb < 1) mb = 1;
  return mb * (1LL << 20) / 8;
}

}  // namespace fftgb

// Same-shape grids run as grouped launches of the uniform fused passes.
struct RgGroup {
  fftgb_shape3 s;
  int nj, r, x;                // pass-A rows per tile, pass-B radix and columns
  std::vector<long long> off;  // first point of each grid
};

struct fftgb_ragged_s {
  std::vector<fftgb_shape3> shapes;
  std::vector<size_t> offset;  // first point of each grid
  size_t points;
  unsigned flags;
  bool persistent;
  bool has_list;  // persistent form: some grids remain in the work list
  std::vector<RgGroup> groups;
  RgExec px;  // persistent form
  // graph-of-plans form, and in the persistent form the grids that are not
  // powers of two: one plan per grid, plan i over grid plan_grid[i]
  std::vector<fftgb_plan> plans;
  std::vector<size_t> plan_grid;
  // cached graph
  cudaGraphExec_t exec;
  const void *g_in;
  void *g_out;
  int g_inv;
  cudaStream_t g_stream;
  unsigned g_gen;  // device-state generation the graph was captured in
};

static bool pow2u(unsigned v) { return v && !(v & (v - 1)); }
static int log2u(unsigned v) {
  int r = 0;
  while ((1u << r) < v) r++;
  return r;
}

// Two passes (kinds 3 and 4, or 3 and z columns) when the grid's shape
// fits the fused tiles of RG_TILE points: nx 32..256, NJ = min(ny, tile/nx)
// rows per pass-A tile (at least 32), R = ny / NJ residues, and for R > 1
// X = tile / (R*nz) pass-B columns with 4 <= X <= nx.
bool fftgb::rg_two_pass_unit(const fftgb_shape3 s, RgUnit *u) {
  const long long tile = ragged_fused_tile_points();
  const int lx = log2u(s.nx), ly = log2u(s.ny), lz = log2u(s.nz);
  if (s.nx < 32 || s.nx > 256 || s.ny < 32 || s.nz < 16 || s.nz > 1024) return false;
  const long long nj = std::min<long long>(s.ny, tile / s.nx);
  if (nj < 32 || !ragged_fused_supported(3, lx, (int)nj)) return false;
  const long long planes = tile / ((long long)s.nx * nj);
  if (planes > s.nz) return false;
  const long long R = s.ny / nj;
  u->npasses = 0;
  u->pass[u->npasses++] = {3, lx, (long long)s.nz, (long long)s.ny, (int)nj};
  (void)ly;
  if (R == 1) {
    u->pass[u->npasses++] = {1, lz, (long long)s.nx * s.ny, (long long)s.nx * s.ny};
    return true;
  }
  const long long X = tile / (R * s.nz);
  if (X < 4 || X > s.nx || !ragged_fused_supported(4, lz, (int)R)) return false;
  u->pass[u->npasses++] = {4, lz, nj * (s.nx / X), (long long)s.nx, (int)R};
  return true;
}

// Shapes that run as grouped uniform passes: pass A k_xy_tma<nx, 64> (R =
// 4), pass B k_rz_tma<256, 4, 8> (and the one-tile kernels of the same
// tiles for unaligned buffers).  Measured on GB300 with the 48-grid 2 GiB
// batch (55 % of its points in 256^3 grids, 15 % in 256 x 256 x 128): 3.61
// ms per forward + inverse against 4.40 with every grid in the work list;
// grouping every shape that has a TMA-fed pass pair (85 % of the points,
// nz = 128 and narrower rows included) took 3.64 ms against 3.61.
static bool rg_grouped_shape(const fftgb_shape3 s, int *nj, int *r, int *x) {
  if (!(s.nz == 256 && s.ny == 256 && (s.nx == 256 || s.nx == 128))) return false;
  if (!fused_xy_tma_available((int)s.nx, 64) || !fused_rz_tma_available(256, 4, 8) ||
      !fused_xy_available((int)s.nx, 64) || !fused_rz_available(256, 4, 8))
    return false;
  *nj = 64, *r = 4, *x = 8;
  return true;
}

static bool rg_grouping() {
  const char *e = getenv("FFTGB_RAGGED_NO_GROUP");
  return !(e && *e == '1');
}

// x rows, then y and z columns, of every grid not in a group (two passes
// where possible; FFTGB_RAGGED_AXES=1 keeps one pass per axis for every grid)
static std::vector<RgUnit> ragged_units(fftgb_ragged r) {
  std::vector<RgUnit> units;
  const char *ax = getenv("FFTGB_RAGGED_AXES");
  const bool axes_only = ax && *ax == '1';
  const bool group = rg_grouping() && !axes_only;
  for (size_t g = 0; g < r->shapes.size(); g++) {
    const fftgb_shape3 s = r->shapes[g];
    if (!pow2u(s.nx) || !pow2u(s.ny) || !pow2u(s.nz)) continue;  // a plan of its own
    int nj = 0, rr = 0, xx = 0;
    if (group && rg_grouped_shape(s, &nj, &rr, &xx)) {
      size_t k = 0;
      while (k < r->groups.size() &&
             !(r->groups[k].s.nx == s.nx && r->groups[k].s.ny == s.ny && r->groups[k].s.nz == s.nz))
        k++;
      if (k == r->groups.size()) r->groups.push_back(RgGroup{s, nj, rr, xx, {}});
      r->groups[k].off.push_back((long long)r->offset[g]);
      continue;
    }
    RgUnit u;
    u.base = (long long)r->offset[g];
    u.points = (long long)s.nx * s.ny * s.nz;
    u.npasses = 0;
    if (!axes_only && rg_two_pass_unit(s, &u)) {
      units.push_back(u);
      continue;
    }
    u.npasses = 0;  // rg_two_pass_unit may have stored pass A before failing
    if (s.nx > 1)
      u.pass[u.npasses++] = {0, log2u(s.nx), (long long)s.ny * s.nz, 1};
    if (s.ny > 1)
      u.pass[u.npasses++] = {1, log2u(s.ny), (long long)s.nx * s.nz, (long long)s.nx};
    if (s.nz > 1)
      u.pass[u.npasses++] = {1, log2u(s.nz), (long long)s.nx * s.ny,
                             (long long)s.nx * s.ny};
    units.push_back(u);
  }
  return units;
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
  r->has_list = false;
  r->exec = NULL;
  r->g_in = NULL;
  r->g_out = NULL;
  r->g_inv = -1;
  r->g_stream = NULL;
  r->g_gen = 0;
  bool any_pow2 = false;
  for (unsigned i = 0; i < count; i++) {
    const fftgb_shape3 s = shapes[i];
    if (s.nx == 0 || s.ny == 0 || s.nz == 0) {
      fftgb_ragged_destroy(r);
      internal_set_err("ragged shapes must have sides of at least 1");
      return FFTGB_EINVAL;
    }
    any_pow2 = any_pow2 || (pow2u(s.nx) && pow2u(s.ny) && pow2u(s.nz));
    r->shapes.push_back(s);
    r->offset.push_back(r->points);
    r->points += (size_t)s.nx * s.ny * s.nz;
  }
  std::vector<RgItem> items;
  int ncounters = 0;
  const char *force_graph = getenv("FFTGB_RAGGED_GRAPH");
  const bool want_persistent =
      (flags & FFTGB_PREC_MASK) == FFTGB_PREC_FP32 &&
      !(force_graph && *force_graph == '1');
  std::vector<RgUnit> units;
  if (want_persistent && any_pow2) units = ragged_units(r);
  if (want_persistent && !units.empty() &&
      rg_build(units, rg_chunk_points(), false, items, &ncounters)) {
    rc = rg_exec_create(items, ncounters, &r->px);
    if (rc) {
      fftgb_ragged_destroy(r);
      internal_set_err("ragged plan allocation failed");
      return rc;
    }
    r->persistent = true;
    r->has_list = true;
  } else if (want_persistent && units.empty() && !r->groups.empty()) {
    r->persistent = true;  // every grid in a group
  } else {
    r->groups.clear();
    r->persistent = false;
  }
  // one plan per grid: every grid in the graph-of-plans form, the grids that
  // are not powers of two (mixed-radix or Bluestein plans) in the persistent
  for (unsigned i = 0; i < count; i++) {
    const fftgb_shape3 s = shapes[i];
    if (r->persistent && pow2u(s.nx) && pow2u(s.ny) && pow2u(s.nz)) continue;
    fftgb_plan p = NULL;
    rc = fftgb_plan_3d(&p, s.nx, s.ny, s.nz, 1, flags);
    if (rc) {
      fftgb_ragged_destroy(r);
      return rc;
    }
    r->plans.push_back(p);
    r->plan_grid.push_back(i);
  }
  *plan = r;
  return FFTGB_OK;
}

extern "C" void fftgb_ragged_destroy(fftgb_ragged r) {
  if (!r) return;
  if (r->exec) cudaGraphExecDestroy(r->exec);
  for (fftgb_plan p : r->plans) fftgb_plan_destroy(p);
  rg_exec_destroy(&r->px);
  delete r;
}

extern "C" size_t fftgb_ragged_points(fftgb_ragged r) {
  return r ? r->points : 0;
}

extern "C" int fftgb_ragged_launches(fftgb_ragged r) {
  if (!r) return 0;
  int n = 0;
  if (r->persistent) {
    n = r->has_list ? 1 : 0;
    for (const RgGroup &g : r->groups)
      n += 2 * (int)((g.off.size() + FUSED_TMA_GRIDS - 1) / FUSED_TMA_GRIDS);
  }
  for (fftgb_plan p : r->plans) n += fftgb_plan_launches(p);
  return n;
}

extern "C" int fftgb_ragged_debug_expire(fftgb_ragged r, unsigned polls) {
  if (!r || polls > (1u << 20)) return FFTGB_EINVAL;
  if (!r->persistent || !r->has_list) return FFTGB_EUNSUP;
  return ragged_expire_wait(r->px.d_counters, r->px.d_status, polls) == cudaSuccess
             ? FFTGB_OK
             : FFTGB_ECUDA;
}

extern "C" int fftgb_ragged_status(fftgb_ragged r) {
  if (!r) return FFTGB_OK;
  int rc = r->persistent && r->has_list ? rg_exec_status(r->px) : FFTGB_OK;
  // the per-grid plans' bounded waits (TMA-fed passes of power-of-two grids)
  for (fftgb_plan p : r->plans) {
    const int st = fftgb_plan_status(p);
    if (st != FFTGB_OK && rc == FFTGB_OK) rc = st;
  }
  if (r->persistent && !r->groups.empty()) {
    // the grouped passes' bounded TMA waits report in the fused-pass status
    const int st = fused_tma_status_and_clear();
    if (st < 0) return FFTGB_ECUDA;
    if (st && rc == FFTGB_OK) {
      internal_set_err("a TMA completion wait of the grouped passes gave up");
      rc = FFTGB_ETIMEOUT;
    }
  }
  return rc;
}

// Passes A and B of one group of same-shape grids (16-byte aligned: the
// TMA-fed kernels over up to FUSED_TMA_GRIDS grids a launch; otherwise the
// one-tile kernels grid by grid, same results).
static int rg_record_group(const RgGroup &g, const float2 *in, float2 *out, int inv,
                           cudaStream_t s) {
  FusedArgs a;
  a.in = in;
  a.out = out;
  a.nx = (int)g.s.nx;
  a.ny = (int)g.s.ny;
  a.nz = (int)g.s.nz;
  a.batch = 1;
  a.tw_x = internal_stage_tw16(log2u(g.s.nx));
  a.tw_j = internal_stage_tw16(log2u((unsigned)g.nj));
  a.tw_y = internal_w_table(log2u(g.s.ny));
  a.tw_z = internal_stage_tw16(log2u(g.s.nz));
  a.scale = 1.0f;
  a.swap_io = inv;
  a.twb = 1;
  FusedArgs b = a;  // pass B in place on the output
  b.in = out;
  const bool aligned = (((uintptr_t)in | (uintptr_t)out) & 15) == 0;
  for (size_t i = 0; i < g.off.size(); i += FUSED_TMA_GRIDS) {
    const int n = (int)std::min<size_t>(FUSED_TMA_GRIDS, g.off.size() - i);
    cudaError_t e;
    if (aligned) {
      e = launch_fused_xy_tma_grids(g.nj, a, &g.off[i], n, s, false);
      if (e == cudaSuccess) e = launch_fused_rz_tma_grids(g.r, g.x, b, &g.off[i], n, s, true);
    } else {
      e = cudaSuccess;
      for (int k = 0; k < n && e == cudaSuccess; k++) {
        FusedArgs ag = a, bg = b;
        ag.in = in + g.off[i + k];
        ag.out = bg.out = out + g.off[i + k];
        bg.in = bg.out;
        e = launch_fused_xy(g.nj, ag, s, false);
        if (e == cudaSuccess) e = launch_fused_rz(g.r, g.x, bg, s, true);
      }
    }
    if (e != cudaSuccess) {
      internal_set_err("grouped pass launch failed");
      return FFTGB_ECUDA;
    }
  }
  return FFTGB_OK;
}

static int record(fftgb_ragged r, const void *d_in, void *d_out, int inv,
                  cudaStream_t cap) {
  int rc = FFTGB_OK;
  if (r->persistent) {
    for (const RgGroup &g : r->groups) {
      rc = rg_record_group(g, (const float2 *)d_in, (float2 *)d_out, inv, cap);
      if (rc) return rc;
    }
    if (r->has_list)
      rc = rg_exec_launch(r->px, (const float2 *)d_in, (float2 *)d_out, inv, 1.0f, cap);
  }
  for (size_t i = 0; i < r->plans.size() && rc == FFTGB_OK; i++) {
    const size_t g = r->plan_grid[i];
    const float2 *src = (const float2 *)d_in + r->offset[g];
    float2 *dst = (float2 *)d_out + r->offset[g];
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
  // the shared tables may have been released by fpga_final since the last
  // call: re-create them, and re-capture if they moved
  int device = 0;
  const int drc = internal_ensure_device(&device);
  if (drc) return drc;
  const unsigned gen = internal_device_generation();
  if (!(r->exec && r->g_in == d_in && r->g_out == d_out && r->g_inv == inv &&
        r->g_stream == s && r->g_gen == gen)) {
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
    r->g_gen = gen;
  }
  if (cudaGraphLaunch(r->exec, s) != cudaSuccess) return FFTGB_ECUDA;
  return FFTGB_OK;
}
