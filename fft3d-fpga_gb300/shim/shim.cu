// shim.cu - C-ABI CUDA shim: device state, twiddle tables, plans, the
// host-buffer transform driver used by the C host library, and the
// device-pointer extension API (fftfpga_ext.h).
//
// Replaces the reference's OpenCL runtime plumbing: global platform/context/
// program/queue state (api/src/fftfpga.c:18-29), per-call queue creation and
// release (fftfpga.c:147-188), per-call buffer creation (api/src/fft3d.c:
// 242-249), binary loading (api/src/opencl_utils.c:141-197) and the SVM
// capability probe (api/src/svm.c:13-52).  Differences by design: state
// persists across calls (stream, device buffers, plans, twiddles), and a
// runtime failure is reported (valid = false / status code) instead of
// exit() (opencl_utils.c:422-440).
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <strings.h>
#include <time.h>
#include <unistd.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "fftfpga.h"
#include "fftfpga_ext.h"
#include "../kernels/fft1d_cluster.cuh"
#include "../kernels/fft3d_fused.cuh"
#include "../kernels/fft_pass.cuh"
#include "shim.h"

using namespace fftgb;

// ------------------------------------------------------------ errors
static thread_local char g_errbuf[512];

static void set_err(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_errbuf, sizeof(g_errbuf), fmt, ap);
  va_end(ap);
}

static bool verbose() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("FFTGB_VERBOSE");
    v = (e && *e && *e != '0') ? 1 : 0;
  }
  return v == 1;
}

#define CK(call)                                                        \
  do {                                                                  \
    cudaError_t e_ = (call);                                            \
    if (e_ != cudaSuccess) {                                            \
      set_err("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),   \
              __FILE__, __LINE__);                                      \
      return FFTGB_ECUDA;                                               \
    }                                                                   \
  } while (0)

static bool is_pow2(unsigned long long v) { return v && !(v & (v - 1)); }
static int ilog2u(unsigned long long v) {
  int r = 0;
  while (v > 1) {
    v >>= 1;
    r++;
  }
  return r;
}

// ------------------------------------------------------------ plans
enum PassKind { P_ROWS, P_COLS, P_COPY, P_XY, P_RZ, P_C1D };

struct Pass {
  PassKind kind;
  int log_l;
  long long count;  // rows or columns
  long long inner;  // column stride
  int out_mode;
  int in_mode;
  int rows_log;
  bool tw4;
  int aux0;  // P_XY: rows per tile (ny / R); P_RZ: R
  int aux1;  // P_RZ: columns per tile
};

struct fftgb_plan_s {
  int rank;
  unsigned n[3];
  unsigned batch;
  unsigned flags;
  size_t points;
  std::vector<Pass> passes;
  bool needs_work;  // intermediate buffer must be distinct from out
  bool inplace_ok;
  float2 *tw4_lo;
  float2 *tw4_hi;
  int tw4_bits;
  float2 *scratch;  // plan-owned work buffer (device-pointer API only)
  fftgb_plan natural_twin;  // natural-order plan used by the adjoint
  // per-pass event profiling
  std::vector<cudaEvent_t> prof_ev;
  int prof_max;
  int prof_count;
  std::vector<std::string> pass_names;
};

// ------------------------------------------------------------ device state
namespace {
struct DeviceState {
  std::recursive_mutex mu;
  bool ready = false;
  int device = -1;
  cudaStream_t stream = nullptr;
  cudaStream_t s_in = nullptr, s_out = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  float2 *tw = nullptr;  // W_L tables for L = 2..4096 at offset L - 2
  float2 *d_in = nullptr, *d_out = nullptr;
  size_t d_cap = 0;  // points
  float2 *h_in = nullptr, *h_out = nullptr;
  size_t h_cap = 0;
  std::map<std::string, fftgb_plan> cache;
  bool svm = false;
  std::string cache_path;
};
DeviceState g;
}  // namespace

static void host_twiddles(std::vector<float2> &v, long long n, long long count,
                          long long step) {
  // W_n^(i*step) for i < count, evaluated in FP64 and rounded once.
  v.resize((size_t)count);
  for (long long i = 0; i < count; i++) {
    const long long m = (i * step) % n;
    double s, c;
    sincos(-2.0 * M_PI * ((double)m / (double)n), &s, &c);
    v[(size_t)i].x = (float)c;
    v[(size_t)i].y = (float)s;
  }
}

static int upload(float2 **dst, const std::vector<float2> &h) {
  CK(cudaMalloc((void **)dst, h.size() * sizeof(float2)));
  CK(cudaMemcpy(*dst, h.data(), h.size() * sizeof(float2),
                cudaMemcpyHostToDevice));
  return FFTGB_OK;
}

// Select the device and set up persistent state (idempotent).
static int ensure_device() {
  if (g.ready) {
    CK(cudaSetDevice(g.device));
    return FFTGB_OK;
  }
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    cudaGetLastError();
    set_err("no CUDA device (%s)", cudaGetErrorString(e));
    return FFTGB_ENODEV;
  }
  g.device = 0;
  CK(cudaSetDevice(g.device));
  CK(cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&g.s_in, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&g.s_out, cudaStreamNonBlocking));
  for (int i = 0; i < 4; i++) CK(cudaEventCreate(&g.ev[i]));
  CK(pass_kernels_init());
  CK(fused_kernels_init());
  CK(cluster1d_init());
  std::vector<float2> all, t;
  for (int l = 1; l <= 12; l++) {
    host_twiddles(t, 1LL << l, 1LL << l, 1);
    all.insert(all.end(), t.begin(), t.end());
  }
  int rc = upload(&g.tw, all);
  if (rc) return rc;
  g.ready = true;
  if (verbose()) fprintf(stderr, "fftgb: device %d ready\n", g.device);
  return FFTGB_OK;
}

static const float2 *tw_table(int log_l) {
  return g.tw + ((1LL << log_l) - 2);
}

static void plan_free(fftgb_plan p) {
  if (!p) return;
  for (cudaEvent_t e : p->prof_ev) cudaEventDestroy(e);
  if (p->tw4_lo) cudaFree(p->tw4_lo);
  if (p->tw4_hi) cudaFree(p->tw4_hi);
  if (p->scratch) cudaFree(p->scratch);
  if (p->natural_twin) plan_free(p->natural_twin);
  delete p;
}

// Two-pass plans for 2D/3D grids (kernels/fft3d_fused.cu).  Leaves
// p->passes empty when no instantiated tile fits the shape.
static int env_int(const char *name) {
  const char *e = getenv(name);
  return (e && *e) ? atoi(e) : 0;
}

// Tile choice: rows per pass-A tile (nj, 0 = largest that fits) and
// columns per pass-B tile (x, 0 = widest available).
static void plan_fused(fftgb_plan p, int force_nj, int force_x) {
  const unsigned nx = p->n[0], ny = p->n[1], nz = p->n[2];
  const long long total = (long long)p->points;
  if (ny < 16) return;
  unsigned nj = 0;
  for (unsigned c = ny; c >= 16; c >>= 1) {
    if (force_nj > 0 && c != (unsigned)force_nj) continue;
    if ((unsigned long long)c * nx <= 16384ULL && fused_xy_available((int)nx, (int)c)) {
      nj = c;
      break;
    }
  }
  if (!nj) return;
  const int R = (int)(ny / nj);
  Pass a = {P_XY, 0, 0, 0, 0, 0, 0, false, (int)nj, 0};
  if (nz == 1) {
    // 2D: pass A, then the radix-R column FFT over the residue rows, which
    // is a strided column pass of length R with stride nx*ny/R
    p->passes.push_back(a);
    if (R > 1) {
      Pass b = {P_COLS, ilog2u((unsigned)R), total / R, (long long)nx * ny / R,
                0, 0, 0, false, 0, 0};
      p->passes.push_back(b);
      p->inplace_ok = false;
    }
    return;
  }
  static const int xs[] = {64, 32, 16, 8, 4};
  for (int X : xs) {
    if (force_x > 0 && X != force_x) continue;
    if ((unsigned)X <= nx && nx % (unsigned)X == 0 &&
        fused_rz_available((int)nz, R, X)) {
      Pass b = {P_RZ, 0, 0, 0, 0, 0, 0, false, R, X};
      p->passes.push_back(a);
      p->passes.push_back(b);
      if (R > 1) p->inplace_ok = false;
      return;
    }
  }
}

static int build_plan(fftgb_plan *out, int rank, unsigned nx, unsigned ny,
                      unsigned nz, unsigned batch, unsigned flags) {
  *out = nullptr;
  if (!is_pow2(nx) || !is_pow2(ny) || !is_pow2(nz) || batch == 0) {
    set_err("sizes must be powers of two and batch >= 1");
    return FFTGB_EINVAL;
  }
  fftgb_plan p = new fftgb_plan_s();
  p->rank = rank;
  p->n[0] = nx;
  p->n[1] = ny;
  p->n[2] = nz;
  p->batch = batch;
  p->flags = flags;
  p->points = (size_t)nx * ny * nz * batch;
  p->needs_work = false;
  p->inplace_ok = true;
  p->tw4_lo = p->tw4_hi = nullptr;
  p->tw4_bits = 0;
  p->scratch = nullptr;
  p->natural_twin = nullptr;
  p->prof_max = 0;
  p->prof_count = 0;
  const long long total = (long long)p->points;
  const bool bitrev = (rank == 1) && (flags & FFTGB_ORDER_BITREV);

  if (rank == 1 && nx > 4096) {
    // four-step: N = L1 * L2, n = n1 + L1*n2, k = k2 + L2*k1
    const int lg = ilog2u(nx);
    if (lg > 24) {
      plan_free(p);
      set_err("1D size %u above 2^24 not supported", nx);
      return FFTGB_EUNSUP;
    }
    const int lg2 = lg / 2, lg1 = lg - lg2;
    const long long L1 = 1LL << lg1, L2 = 1LL << lg2;
    const int bits = (lg + 1) / 2;
    std::vector<float2> lo, hi;
    host_twiddles(lo, nx, 1LL << bits, 1);
    host_twiddles(hi, nx, (long long)nx >> bits, 1LL << bits);
    int rc = upload(&p->tw4_lo, lo);
    if (!rc) rc = upload(&p->tw4_hi, hi);
    if (rc) {
      plan_free(p);
      return rc;
    }
    p->tw4_bits = bits;
    int cl1 = 0, cl2 = 0;
    if (env_int("FFTGB_NO_CLUSTER") != 1 &&
        cluster1d_available((int)nx, &cl1, &cl2)) {
      // one pass: the four-step transpose goes through distributed shared
      // memory of a thread-block cluster (kernels/fft1d_cluster.cu)
      Pass c = {P_C1D, 0, (long long)batch, 0, bitrev ? 1 : 0, 0, 0, true, cl1,
                cl2};
      p->passes.push_back(c);
    } else {
      Pass a = {P_COLS, lg2, batch * L1, L1, bitrev ? 0 : 1, 0, 0, true};
      p->passes.push_back(a);
    }
    if (!p->passes.empty() && p->passes[0].kind == P_C1D) {
      // done
    } else if (bitrev) {
      Pass b = {P_ROWS, lg1, batch * L2, 0, 2, 0, lg2, false};
      p->passes.push_back(b);
      p->needs_work = true;
    } else {
      Pass b = {P_COLS, lg1, batch * L2, L2, 0, 0, 0, false};
      p->passes.push_back(b);
    }
    p->inplace_ok = p->passes[0].kind == P_C1D;
  } else {
    if (nx > 4096 || ny > 4096 || nz > 4096) {
      plan_free(p);
      set_err("axis length above 4096 not supported for rank %d", rank);
      return FFTGB_EUNSUP;
    }
    // FFTGB_NO_FUSED=1 selects the per-axis plan; FFTGB_FUSED_NJ and
    // FFTGB_FUSED_X pin the fused tile shape (tuning overrides)
    if (env_int("FFTGB_NO_FUSED") != 1 && rank >= 2)
      plan_fused(p, env_int("FFTGB_FUSED_NJ"), env_int("FFTGB_FUSED_X"));
    if (p->passes.empty()) {
      if (nx > 1) {
        Pass a = {P_ROWS, ilog2u(nx), total / nx, 0, bitrev ? 1 : 0, 0, 0,
                  false, 0, 0};
        p->passes.push_back(a);
      }
      if (ny > 1) {
        Pass b = {P_COLS, ilog2u(ny), total / ny, (long long)nx, 0, 0, 0, false,
                  0, 0};
        p->passes.push_back(b);
      }
      if (nz > 1) {
        Pass c = {P_COLS, ilog2u(nz), total / nz, (long long)nx * ny, 0, 0, 0,
                  false, 0, 0};
        p->passes.push_back(c);
      }
    }
    if (p->passes.empty()) {
      Pass c = {P_COPY, 0, total, 0, 0, 0, 0, false, 0, 0};
      p->passes.push_back(c);
    }
  }
  for (const Pass &ps : p->passes) {
    char nm[48];
    if (ps.kind == P_COPY)
      snprintf(nm, sizeof(nm), "memcpy");
    else if (ps.kind == P_XY)
      snprintf(nm, sizeof(nm), "k_xy<%u,%d>", p->n[0], ps.aux0);
    else if (ps.kind == P_C1D)
      snprintf(nm, sizeof(nm), "k_1d_cluster<%d,%d>", ps.aux0, ps.aux1);
    else if (ps.kind == P_RZ)
      snprintf(nm, sizeof(nm), "k_rz<%u,%d,%d>", p->n[2], ps.aux0, ps.aux1);
    else
      snprintf(nm, sizeof(nm), "%s<%d>", ps.kind == P_ROWS ? "k_rows" : "k_cols",
               1 << ps.log_l);
    p->pass_names.push_back(nm);
  }
  *out = p;
  return FFTGB_OK;
}

// Launch the plan's passes: in -> [work ...] -> out.
static int run_passes(fftgb_plan p, const float2 *in, float2 *out, float2 *work,
                      int inverse, float scale, cudaStream_t s) {
  const int np = (int)p->passes.size();
  cudaEvent_t *ev = nullptr;
  if (p->prof_count < p->prof_max) {
    ev = &p->prof_ev[(size_t)p->prof_count * (size_t)(np + 1)];
    p->prof_count++;
  }
  for (int i = 0; i < np; i++) {
    const Pass &ps = p->passes[(size_t)i];
    if (ev) cudaEventRecord(ev[i], s);
    const float2 *src = (i == 0) ? in : work;
    float2 *dst = (i == np - 1) ? out : work;
    const float sc = (i == np - 1) ? scale : 1.0f;
    cudaError_t e = cudaSuccess;
    if (ps.kind == P_ROWS) {
      RowsArgs a;
      a.in = src;
      a.out = dst;
      a.nrows = ps.count;
      a.tw = tw_table(ps.log_l);
      a.scale = sc;
      a.swap_io = inverse ? 1 : 0;
      a.in_mode = ps.in_mode;
      a.out_mode = ps.out_mode;
      a.rows_log = ps.rows_log;
      e = launch_rows(ps.log_l, a, s);
    } else if (ps.kind == P_COLS) {
      ColsArgs a;
      a.in = src;
      a.out = dst;
      a.ncols = ps.count;
      a.inner = ps.inner;
      a.tw = tw_table(ps.log_l);
      a.tw4_lo = ps.tw4 ? p->tw4_lo : nullptr;
      a.tw4_hi = ps.tw4 ? p->tw4_hi : nullptr;
      a.tw4_bits = p->tw4_bits;
      a.scale = sc;
      a.swap_io = inverse ? 1 : 0;
      a.out_mode = ps.out_mode;
      e = launch_cols(ps.log_l, a, s);
    } else if (ps.kind == P_C1D) {
      C1dArgs a;
      a.in = src;
      a.out = dst;
      a.count = ps.count;
      a.tw_a = tw_table(ilog2u((unsigned)ps.aux1));
      a.tw_b = tw_table(ilog2u((unsigned)ps.aux0));
      a.tw4_lo = p->tw4_lo;
      a.tw4_hi = p->tw4_hi;
      a.tw4_bits = p->tw4_bits;
      a.bitrev = ps.out_mode;
      a.scale = sc;
      a.swap_io = inverse ? 1 : 0;
      e = launch_cluster1d((int)p->n[0], a, s);
    } else if (ps.kind == P_XY || ps.kind == P_RZ) {
      FusedArgs a;
      a.in = src;
      a.out = dst;
      a.nx = (int)p->n[0];
      a.ny = (int)p->n[1];
      a.nz = (int)p->n[2];
      a.batch = p->batch;
      a.tw_x = tw_table(ilog2u(p->n[0]));
      a.tw_y = tw_table(ilog2u(p->n[1]));
      a.tw_z = p->n[2] > 1 ? tw_table(ilog2u(p->n[2])) : nullptr;
      a.tw_j = ps.kind == P_XY ? tw_table(ilog2u((unsigned)ps.aux0)) : nullptr;
      a.scale = sc;
      a.swap_io = inverse ? 1 : 0;
      e = ps.kind == P_XY ? launch_fused_xy(ps.aux0, a, s)
                          : launch_fused_rz(ps.aux0, ps.aux1, a, s);
    } else {
      if (scale != 1.0f) {
        set_err("scaled size-1 transforms are not supported");
        return FFTGB_EUNSUP;
      }
      if (src != dst)
        e = cudaMemcpyAsync(dst, src, (size_t)ps.count * sizeof(float2),
                            cudaMemcpyDeviceToDevice, s);
    }
    if (e != cudaSuccess) {
      set_err("pass %d launch failed: %s", i, cudaGetErrorString(e));
      return FFTGB_ECUDA;
    }
  }
  if (ev) cudaEventRecord(ev[np], s);
  return FFTGB_OK;
}

static int ensure_scratch(fftgb_plan p) {
  if (p->needs_work && !p->scratch)
    CK(cudaMalloc((void **)&p->scratch, p->points * sizeof(float2)));
  return FFTGB_OK;
}

// ------------------------------------------------------------ host buffers
static int ensure_dev_buffers(size_t points) {
  if (points <= g.d_cap) return FFTGB_OK;
  if (g.d_in) cudaFree(g.d_in);
  if (g.d_out) cudaFree(g.d_out);
  g.d_in = g.d_out = nullptr;
  g.d_cap = 0;
  cudaError_t e1 = cudaMalloc((void **)&g.d_in, points * sizeof(float2));
  cudaError_t e2 = cudaMalloc((void **)&g.d_out, points * sizeof(float2));
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    if (g.d_in) cudaFree(g.d_in);
    if (g.d_out) cudaFree(g.d_out);
    g.d_in = g.d_out = nullptr;
    cudaGetLastError();
    set_err("device allocation of %zu points failed", points);
    return FFTGB_ENOMEM;
  }
  g.d_cap = points;
  return FFTGB_OK;
}

static int ensure_host_staging(size_t points) {
  if (points <= g.h_cap) return FFTGB_OK;
  if (g.h_in) cudaFreeHost(g.h_in);
  if (g.h_out) cudaFreeHost(g.h_out);
  g.h_in = g.h_out = nullptr;
  g.h_cap = 0;
  cudaError_t e1 = cudaHostAlloc((void **)&g.h_in, points * sizeof(float2),
                                 cudaHostAllocMapped | cudaHostAllocPortable);
  cudaError_t e2 = cudaHostAlloc((void **)&g.h_out, points * sizeof(float2),
                                 cudaHostAllocMapped | cudaHostAllocPortable);
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    if (g.h_in) cudaFreeHost(g.h_in);
    if (g.h_out) cudaFreeHost(g.h_out);
    g.h_in = g.h_out = nullptr;
    cudaGetLastError();
    set_err("pinned host allocation of %zu points failed", points);
    return FFTGB_ENOMEM;
  }
  g.h_cap = points;
  return FFTGB_OK;
}

static int cached_plan(fftgb_plan *out, unsigned nx, unsigned ny, unsigned nz,
                       unsigned batch, unsigned flags) {
  char key[96];
  snprintf(key, sizeof(key), "%u,%u,%u,%u,%u", nx, ny, nz, batch, flags);
  auto it = g.cache.find(key);
  if (it != g.cache.end()) {
    *out = it->second;
    return FFTGB_OK;
  }
  const int rank = nz > 1 ? 3 : (ny > 1 ? 2 : 1);
  int rc = build_plan(out, rank, nx, ny, nz, batch, flags);
  if (rc) return rc;
  g.cache[key] = *out;
  return FFTGB_OK;
}

static double now_ms() {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec * 1e3 + (double)ts.tv_nsec * 1e-6;
}

static double ev_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) return 0.0;
  return (double)ms;
}

static int run_copy(fftgb_plan p, const float2 *inp, float2 *out, bool inv,
                    fpga_t *t) {
  const size_t bytes = p->points * sizeof(float2);
  int rc = ensure_dev_buffers(p->points);
  if (rc) return rc;
  float2 *work = p->needs_work ? g.d_in : g.d_out;
  cudaStream_t s = g.stream;
  CK(cudaEventRecord(g.ev[0], s));
  CK(cudaMemcpyAsync(g.d_in, inp, bytes, cudaMemcpyHostToDevice, s));
  CK(cudaEventRecord(g.ev[1], s));
  rc = run_passes(p, g.d_in, g.d_out, work, inv, 1.0f, s);
  if (rc) return rc;
  CK(cudaEventRecord(g.ev[2], s));
  CK(cudaMemcpyAsync(out, g.d_out, bytes, cudaMemcpyDeviceToHost, s));
  CK(cudaEventRecord(g.ev[3], s));
  CK(cudaStreamSynchronize(s));
  t->pcie_write_t = ev_ms(g.ev[0], g.ev[1]);
  t->exec_t = ev_ms(g.ev[1], g.ev[2]);
  t->pcie_read_t = ev_ms(g.ev[2], g.ev[3]);
  return FFTGB_OK;
}

// Per-grid copies overlapped with compute, as the reference's buffer
// rotation does (api/src/fft3d.c:551-705); exec_t is wall time.
static int run_pipeline(unsigned nx, unsigned ny, unsigned nz, unsigned batch,
                        unsigned flags, const float2 *inp, float2 *out,
                        bool inv, fpga_t *t) {
  fftgb_plan p1 = nullptr;
  int rc = cached_plan(&p1, nx, ny, nz, 1, flags);
  if (rc) return rc;
  const size_t grid = p1->points;
  rc = ensure_dev_buffers(grid * batch);
  if (rc) return rc;
  std::vector<cudaEvent_t> ev_in(batch), ev_done(batch);
  for (unsigned i = 0; i < batch; i++) {
    CK(cudaEventCreateWithFlags(&ev_in[i], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev_done[i], cudaEventDisableTiming));
  }
  const double t0 = now_ms();
  const size_t bytes = grid * sizeof(float2);
  int status = FFTGB_OK;
  for (unsigned i = 0; i < batch && status == FFTGB_OK; i++) {
    float2 *din = g.d_in + grid * i, *dout = g.d_out + grid * i;
    if (cudaMemcpyAsync(din, inp + grid * i, bytes, cudaMemcpyHostToDevice,
                        g.s_in) != cudaSuccess ||
        cudaEventRecord(ev_in[i], g.s_in) != cudaSuccess ||
        cudaStreamWaitEvent(g.stream, ev_in[i], 0) != cudaSuccess) {
      set_err("pipelined copy-in failed");
      status = FFTGB_ECUDA;
      break;
    }
    status = run_passes(p1, din, dout, p1->needs_work ? din : dout, inv, 1.0f,
                        g.stream);
    if (status) break;
    if (cudaEventRecord(ev_done[i], g.stream) != cudaSuccess ||
        cudaStreamWaitEvent(g.s_out, ev_done[i], 0) != cudaSuccess ||
        cudaMemcpyAsync(out + grid * i, dout, bytes, cudaMemcpyDeviceToHost,
                        g.s_out) != cudaSuccess) {
      set_err("pipelined copy-out failed");
      status = FFTGB_ECUDA;
    }
  }
  cudaError_t e1 = cudaStreamSynchronize(g.s_in);
  cudaError_t e2 = cudaStreamSynchronize(g.stream);
  cudaError_t e3 = cudaStreamSynchronize(g.s_out);
  t->exec_t = now_ms() - t0;
  for (unsigned i = 0; i < batch; i++) {
    cudaEventDestroy(ev_in[i]);
    cudaEventDestroy(ev_done[i]);
  }
  if (status) return status;
  if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) {
    set_err("pipelined transform failed: %s",
            cudaGetErrorString(e2 != cudaSuccess ? e2 : (e1 ? e1 : e3)));
    return FFTGB_ECUDA;
  }
  return FFTGB_OK;
}

// Kernels read the input from, and write the output to, device-mapped
// pinned host staging; intermediate passes stay in HBM.
static int run_svm(fftgb_plan p, const float2 *inp, float2 *out, bool inv,
                   fpga_t *t) {
  const size_t bytes = p->points * sizeof(float2);
  int rc = ensure_host_staging(p->points);
  if (!rc) rc = ensure_dev_buffers(p->points);
  if (rc) return rc;
  double t0 = now_ms();
  memcpy(g.h_in, inp, bytes);
  t->svm_copyin_t = now_ms() - t0;
  float2 *din = nullptr, *dout = nullptr;
  CK(cudaHostGetDevicePointer((void **)&din, g.h_in, 0));
  CK(cudaHostGetDevicePointer((void **)&dout, g.h_out, 0));
  cudaStream_t s = g.stream;
  CK(cudaEventRecord(g.ev[0], s));
  rc = run_passes(p, din, dout, g.d_out, inv, 1.0f, s);
  if (rc) return rc;
  CK(cudaEventRecord(g.ev[1], s));
  CK(cudaStreamSynchronize(s));
  t->exec_t = ev_ms(g.ev[0], g.ev[1]);
  t0 = now_ms();
  memcpy(out, g.h_out, bytes);
  t->svm_copyout_t = now_ms() - t0;
  return FFTGB_OK;
}

// ------------------------------------------------------------ shim C API
extern "C" int fftgb_shim_initialize(const char *platform_name,
                                     const char *path, bool use_svm) {
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  if (path == NULL || strlen(path) == 0) return -1;
  if (platform_name == NULL || strlen(platform_name) == 0) return -2;
  // case-insensitive substring search of the argument inside the platform
  // name, as findPlatform does (api/src/opencl_utils.c:50-80)
  std::string arg(platform_name);
  for (auto &ch : arg) ch = (char)tolower((unsigned char)ch);
  bool match = std::string("nvidia cuda").find(arg) != std::string::npos;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess) cudaGetLastError();
  if (!match && e == cudaSuccess && count > 0) {
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, 0) == cudaSuccess) {
      std::string name(prop.name);
      for (auto &ch : name) ch = (char)tolower((unsigned char)ch);
      match = name.find(arg) != std::string::npos;
    }
  }
  if (!match) return -2;
  if (e != cudaSuccess || count == 0) return -3;
  if (ensure_device() != FFTGB_OK) return -3;
  if (use_svm) {
    int pageable = 0, mapped = 0;
    cudaDeviceGetAttribute(&mapped, cudaDevAttrCanMapHostMemory, g.device);
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, g.device);
    if (!mapped) return -5;
    g.svm = true;
    if (verbose())
      fprintf(stderr, "fftgb: host-mapped staging enabled (pageable=%d)\n",
              pageable);
  } else {
    g.svm = false;
  }
  if (access(path, R_OK) != 0) return -4;
  g.cache_path = path;
  return 0;
}

extern "C" void fftgb_shim_final(void) {
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  if (!g.ready) {
    g.svm = false;
    return;
  }
  cudaSetDevice(g.device);
  cudaDeviceSynchronize();
  for (auto &kv : g.cache) plan_free(kv.second);
  g.cache.clear();
  if (g.d_in) cudaFree(g.d_in);
  if (g.d_out) cudaFree(g.d_out);
  g.d_in = g.d_out = nullptr;
  g.d_cap = 0;
  if (g.h_in) cudaFreeHost(g.h_in);
  if (g.h_out) cudaFreeHost(g.h_out);
  g.h_in = g.h_out = nullptr;
  g.h_cap = 0;
  if (g.tw) cudaFree(g.tw);
  g.tw = nullptr;
  for (int i = 0; i < 4; i++) {
    if (g.ev[i]) cudaEventDestroy(g.ev[i]);
    g.ev[i] = nullptr;
  }
  if (g.stream) cudaStreamDestroy(g.stream);
  if (g.s_in) cudaStreamDestroy(g.s_in);
  if (g.s_out) cudaStreamDestroy(g.s_out);
  g.stream = g.s_in = g.s_out = nullptr;
  g.svm = false;
  g.ready = false;
}

extern "C" int fftgb_shim_svm_enabled(void) { return g.svm ? 1 : 0; }

extern "C" fpga_t fftgb_shim_run(unsigned nx, unsigned ny, unsigned nz,
                                 unsigned batch, unsigned flags,
                                 const float2 *inp, float2 *out, bool inv,
                                 int mode) {
  fpga_t t;
  memset(&t, 0, sizeof(t));
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  if (ensure_device() != FFTGB_OK) return t;
  int rc;
  if (mode == FFTGB_RUN_PIPELINE) {
    rc = run_pipeline(nx, ny, nz, batch, flags, inp, out, inv, &t);
  } else {
    fftgb_plan p = nullptr;
    rc = cached_plan(&p, nx, ny, nz, batch, flags);
    if (!rc) rc = (mode == FFTGB_RUN_SVM) ? run_svm(p, inp, out, inv, &t)
                                          : run_copy(p, inp, out, inv, &t);
  }
  if (rc != FFTGB_OK) {
    if (verbose()) fprintf(stderr, "fftgb: %s\n", g_errbuf);
    fpga_t bad;
    memset(&bad, 0, sizeof(bad));
    return bad;
  }
  t.valid = true;
  return t;
}

// ------------------------------------------------------------ ext API
static int plan_entry(fftgb_plan *plan, int rank, unsigned nx, unsigned ny,
                      unsigned nz, unsigned batch, unsigned flags) {
  if (plan == NULL) {
    set_err("plan pointer is NULL");
    return FFTGB_EINVAL;
  }
  *plan = nullptr;
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  int rc = ensure_device();
  if (rc) return rc;
  if ((flags & FFTGB_PREC_MASK) != FFTGB_PREC_FP32) {
    set_err("precision mode 0x%x not available for this plan", flags);
    return FFTGB_EUNSUP;
  }
  rc = build_plan(plan, rank, nx, ny, nz, batch, flags);
  if (rc) return rc;
  rc = ensure_scratch(*plan);
  if (rc) {
    plan_free(*plan);
    *plan = nullptr;
  }
  return rc;
}

extern "C" int fftgb_plan_1d(fftgb_plan *plan, unsigned n, unsigned batch,
                             unsigned flags) {
  return plan_entry(plan, 1, n, 1, 1, batch, flags);
}
extern "C" int fftgb_plan_2d(fftgb_plan *plan, unsigned nx, unsigned ny,
                             unsigned batch, unsigned flags) {
  return plan_entry(plan, 2, nx, ny, 1, batch, flags & ~FFTGB_ORDER_BITREV);
}
extern "C" int fftgb_plan_3d(fftgb_plan *plan, unsigned nx, unsigned ny,
                             unsigned nz, unsigned batch, unsigned flags) {
  return plan_entry(plan, 3, nx, ny, nz, batch, flags & ~FFTGB_ORDER_BITREV);
}

extern "C" void fftgb_plan_destroy(fftgb_plan plan) {
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  plan_free(plan);
}

extern "C" size_t fftgb_plan_points(fftgb_plan plan) {
  return plan ? plan->points : 0;
}

extern "C" int fftgb_plan_launches(fftgb_plan plan) {
  return plan ? (int)plan->passes.size() : 0;
}

extern "C" int fftgb_plan_inplace_ok(fftgb_plan plan) {
  return (plan && plan->inplace_ok) ? 1 : 0;
}

static int check_io(fftgb_plan plan, const void *d_in, void *d_out) {
  if (!plan || !d_in || !d_out) {
    set_err("NULL plan or buffer");
    return FFTGB_EINVAL;
  }
  const char *a = (const char *)d_in, *b = (const char *)d_out;
  const size_t bytes = plan->points * sizeof(float2);
  if (a == b) {
    if (!plan->inplace_ok) {
      set_err("this plan cannot run in place");
      return FFTGB_EINVAL;
    }
  } else if (a < b + bytes && b < a + bytes) {
    set_err("input and output overlap partially");
    return FFTGB_EINVAL;
  }
  return FFTGB_OK;
}

extern "C" int fftgb_exec(fftgb_plan plan, const void *d_in, void *d_out,
                          int inverse, float scale, void *stream) {
  int rc = check_io(plan, d_in, d_out);
  if (rc) return rc;
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  // fpga_final may have released the shared twiddle table since the plan
  // was made; re-create device state before any launch reads it
  rc = ensure_device();
  if (rc) return rc;
  float2 *out = (float2 *)d_out;
  float2 *work = plan->needs_work ? plan->scratch : out;
  return run_passes(plan, (const float2 *)d_in, out, work, inverse, scale,
                    (cudaStream_t)stream);
}

extern "C" int fftgb_exec_adjoint(fftgb_plan plan, const void *d_in,
                                  void *d_out, int inverse, float scale,
                                  void *stream) {
  int rc = check_io(plan, d_in, d_out);
  if (rc) return rc;
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  rc = ensure_device();
  if (rc) return rc;
  const bool bitrev = (plan->rank == 1) && (plan->flags & FFTGB_ORDER_BITREV);
  // adjoint(forward) = unnormalised inverse and vice versa (the DFT matrix
  // is symmetric); a bit-reversed output order becomes a bit-reversed load.
  const int dir = inverse ? 0 : 1;
  if (!bitrev)
    return fftgb_exec(plan, d_in, d_out, dir, scale, stream);
  if (d_in == d_out) {
    set_err("adjoint of a bit-reversed plan cannot run in place");
    return FFTGB_EINVAL;
  }
  const unsigned n = plan->n[0];
  if (n <= 4096) {
    RowsArgs a;
    a.in = (const float2 *)d_in;
    a.out = (float2 *)d_out;
    a.nrows = plan->batch;
    a.tw = tw_table(ilog2u(n));
    a.scale = scale;
    a.swap_io = dir;
    a.in_mode = 1;
    a.out_mode = 0;
    a.rows_log = 0;
    cudaError_t e = (n == 1) ? cudaMemcpyAsync(d_out, d_in, plan->points * 8,
                                               cudaMemcpyDeviceToDevice,
                                               (cudaStream_t)stream)
                             : launch_rows(ilog2u(n), a, (cudaStream_t)stream);
    if (e != cudaSuccess) {
      set_err("adjoint launch failed: %s", cudaGetErrorString(e));
      return FFTGB_ECUDA;
    }
    return FFTGB_OK;
  }
  if (!plan->natural_twin) {
    rc = build_plan(&plan->natural_twin, 1, n, 1, 1, plan->batch,
                    FFTGB_ORDER_NATURAL);
    if (rc) return rc;
  }
  // un-bit-reverse into the plan scratch, then the natural-order transform
  if (!plan->scratch)
    CK(cudaMalloc((void **)&plan->scratch, plan->points * sizeof(float2)));
  cudaError_t e = launch_bitrev_gather((const float2 *)d_in, plan->scratch, n,
                                       ilog2u(n), plan->batch,
                                       (cudaStream_t)stream);
  if (e != cudaSuccess) {
    set_err("adjoint gather failed: %s", cudaGetErrorString(e));
    return FFTGB_ECUDA;
  }
  return run_passes(plan->natural_twin, plan->scratch, (float2 *)d_out,
                    (float2 *)d_out, dir, scale, (cudaStream_t)stream);
}

extern "C" int fftgb_profile_begin(fftgb_plan plan, int max_execs) {
  if (!plan || max_execs < 1) return FFTGB_EINVAL;
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  int rc = ensure_device();
  if (rc) return rc;
  const size_t need = (size_t)max_execs * (plan->passes.size() + 1);
  while (plan->prof_ev.size() < need) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    plan->prof_ev.push_back(e);
  }
  plan->prof_max = max_execs;
  plan->prof_count = 0;
  return FFTGB_OK;
}

extern "C" int fftgb_profile_end(fftgb_plan plan, float *ms_per_pass, int npass,
                                 int *nexec) {
  if (!plan || !ms_per_pass) return FFTGB_EINVAL;
  const int np = (int)plan->passes.size();
  for (int i = 0; i < npass; i++) ms_per_pass[i] = 0.f;
  const int n = plan->prof_count;
  for (int x = 0; x < n; x++) {
    cudaEvent_t *ev = &plan->prof_ev[(size_t)x * (size_t)(np + 1)];
    CK(cudaEventSynchronize(ev[np]));
    for (int i = 0; i < np && i < npass; i++) {
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]));
      ms_per_pass[i] += ms;
    }
  }
  if (nexec) *nexec = n;
  plan->prof_max = 0;
  plan->prof_count = 0;
  return FFTGB_OK;
}

extern "C" const char *fftgb_plan_pass_name(fftgb_plan plan, int i) {
  if (!plan || i < 0 || i >= (int)plan->pass_names.size()) return "";
  return plan->pass_names[(size_t)i].c_str();
}

extern "C" const char *fftgb_last_error(void) { return g_errbuf; }

extern "C" const char *fftgb_version(void) { return "fftgb 0.1 (sm_103a)"; }
