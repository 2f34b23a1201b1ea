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

#include <algorithm>
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
#include "../kernels/fft3d_cluster.cuh"
#include "../kernels/spectral.cuh"
#include "../kernels/fft3d_fused.cuh"
#include "../kernels/fft_tc.cuh"
#include "../kernels/fft_pass.cuh"
#include "../kernels/fft_blue.cuh"
#include "../kernels/fft_mix.cuh"
#include "shim.h"

#include "tables.h"
#include "../kernels/fft_core.cuh"

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
enum PassKind { P_ROWS, P_COLS, P_COPY, P_XY, P_RZ, P_C1D, P_BLUE, P_C3D, P_MIX };

enum VariantKind { V_DEFAULT = 0, V_AXIS, V_FUSED, V_CLUSTER, V_FOURSTEP, V_NONPOW2 };
struct Variant {
  int kind;
  int nj;  // V_FUSED: rows per pass-A tile
  int x;   // V_FUSED: columns per pass-B tile; V_CLUSTER: CTAs per cluster (0: default);
           // V_AXIS: 8 = y-blocked intermediate layout (3D)
  int pipe = 0;  // V_FUSED: pass A (16) / pass B (32) as persistent kernels fed by
                 // TMA tensor copies; 8: the one-tile passes with 8 points per
                 // thread (where built)
};

struct Pass {
  PassKind kind;
  int log_l;
  long long count;  // rows or columns
  long long inner;  // column stride
  int out_mode;
  int in_mode;
  int rows_log;
  bool tw4;
  int aux0;  // P_XY: rows per tile (ny / R); P_RZ: R; P_COLS: 2 = TMA-fed
  int aux1;  // P_RZ: columns per tile
  int tc;    // P_ROWS/P_COLS: 0 FP32, 1 split-FP16 / 2 split-BF16 tensor cores
  int blk = -1;  // P_COLS: >= 0 reads the y-blocked layout (log2 nz; TMA only)
  int ept = 16;  // P_XY/P_RZ one-tile kernels: points per thread (16 or 8)
};

// Plans built for the host-buffer calls (their work buffer is the input's
// device copy): no y-blocked per-axis plan, whose first pass cannot run in
// place.  A private bit of the plan flags, never set by callers.
#define FFTGB_FLAG_NATURAL_AXES 0x40000000u

// Tensor-core mode of the plan flags: 0 (FP32), 1 (split FP16), 2 (split BF16).
static int tc_mode(unsigned flags) {
  switch (flags & FFTGB_PREC_MASK) {
    case FFTGB_PREC_TC_FP16: return 1;
    case FFTGB_PREC_TC_BF16: return 2;
    default: return 0;
  }
}

struct fftgb_plan_s {
  int rank;
  unsigned n[3];
  unsigned batch;
  unsigned flags;
  size_t points;
  std::vector<Pass> passes;
  bool needs_work;  // intermediate buffer must be distinct from out
  bool inplace_ok;
  bool twb;  // 3D fused plans: pass B applies pass A's y twiddle (FusedArgs::twb)
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
  struct Variant variant;
  float2 *blue_w[3] = {nullptr, nullptr, nullptr};  // P_BLUE per axis: chirp
  float2 *blue_h[3] = {nullptr, nullptr, nullptr};  //   and filter spectrum / M
  float2 *mix_w[3] = {nullptr, nullptr, nullptr};   // P_MIX per axis: W_n table
  int mix_nst[3] = {0, 0, 0};                       //   stage count
  int mix_rad[3][MIX_MAXST] = {};                   //   and stage radices
};

// ------------------------------------------------------------ device state
namespace {
struct DeviceState {
  std::recursive_mutex mu;
  bool ready = false;
  unsigned generation = 0;  // bumped whenever the shared tables are (re)created
  int device = -1;
  cudaStream_t stream = nullptr;
  cudaStream_t s_in = nullptr, s_out = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  std::vector<cudaEvent_t> cev;  // chunked copy pipeline: 6 per chunk
  float2 *tw = nullptr;  // W_L tables for L = 2..4096 at offset L - 2
  // Stockham stage tables for E = 8 ([0]) and E = 16 ([1]), per log2 L
  float2 *tws[2] = {nullptr, nullptr};
  size_t tws_off[2][13] = {};
  float2 *d_in = nullptr, *d_out = nullptr;
  size_t d_cap = 0;  // points
  float2 *h_in = nullptr, *h_out = nullptr;
  size_t h_cap = 0;
  std::map<std::string, fftgb_plan> cache;
  bool svm = false;
  std::string cache_path;
  // tuning cache: shape key -> variant, persisted as JSON at tune_path
  std::map<std::string, std::string> tune;
  std::string tune_path;
  bool tune_loaded = false;
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
  CK(fused_tma_init());
  CK(cols_tma_init());
  CK(blue_kernels_init());
  CK(mix_kernels_init());
  CK(cluster1d_init());
  CK(cluster3d_init());
  CK(tc_kernels_init());
  std::vector<float2> all, t;
  for (int l = 1; l <= 12; l++) {
    host_twiddles(t, 1LL << l, 1LL << l, 1);
    all.insert(all.end(), t.begin(), t.end());
  }
  int rc = upload(&g.tw, all);
  if (rc) return rc;
  for (int e = 0; e < 2; e++) {
    std::vector<float2> st;
    for (int l = 1; l <= 12; l++) {
      g.tws_off[e][l] = st.size();
      stage_table(st, 1 << l, e ? 16 : 8);
    }
    rc = upload(&g.tws[e], st);
    if (rc) return rc;
  }
  g.ready = true;
  g.generation++;
  if (verbose()) fprintf(stderr, "fftgb: device %d ready\n", g.device);
  return FFTGB_OK;
}

// Stage table of Stock<2^log_l, e> (e = points per thread).
static const float2 *stage_tw(int log_l, int e) {
  const int i = e >= 16 ? 1 : 0;
  return g.tws[i] + g.tws_off[i][log_l];
}

// Stage table of the per-axis kernels' plan for length 2^log_l.
static const float2 *axis_tw(int log_l) {
  return stage_tw(log_l, default_e(1 << log_l));
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
  for (int a = 0; a < 3; a++) {
    if (p->blue_w[a]) cudaFree(p->blue_w[a]);
    if (p->blue_h[a]) cudaFree(p->blue_h[a]);
    if (p->mix_w[a]) cudaFree(p->mix_w[a]);
  }
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
static void plan_fused(fftgb_plan p, int force_nj, int force_x, int pipe) {
  const unsigned nx = p->n[0], ny = p->n[1], nz = p->n[2];
  const long long total = (long long)p->points;
  if (ny < (nz == 1 ? 2u : 16u)) return;
  unsigned nj = 0;
  // 2D tiles may be as short as 2 rows (pass B is then a long column FFT);
  // 3D needs at least 16 (pass B's radix R = ny / nj is at most 16)
  const unsigned cmin = nz == 1 ? 2 : 16;
  for (unsigned c = ny; c >= cmin; c >>= 1) {
    if (force_nj > 0 && c != (unsigned)force_nj) continue;
    if ((unsigned long long)c * nx <= 16384ULL && fused_xy_available((int)nx, (int)c)) {
      nj = c;
      break;
    }
  }
  if (!nj) return;
  const int R = (int)(ny / nj);
  // out_mode 3: persistent, tiles copied in by TMA
  const int pa = (pipe & 16) && fused_xy_tma_available((int)nx, (int)nj) ? 3 : 0;
  Pass a = {P_XY, 0, 0, 0, pa, 0, 0, false, (int)nj, 0};
  if (nz == 1) {
    // 2D: pass A, then the radix-R column FFT over the residue rows, which
    // is a strided column pass of length R with stride nx*ny/R
    p->passes.push_back(a);
    if (R > 1) {
      Pass b = {P_COLS, ilog2u((unsigned)R), total / R, (long long)nx * ny / R,
                0, 0, 0, false, 0, 0};
      // up to R = 128 the y twiddle W_ny^(r*k1) goes with the column pass's
      // loads (input r of column c = k1*nx + x: exponent r * (c >> log2
      // nx)), taking a table read and a multiply per point out of the
      // issue-bound pass A: 1024^2 x 64 0.393 against 0.395 ms; a 512-point
      // column pass loses more than pass A gains (2048^2 x 16: 0.435
      // against 0.431 ms).  FFTGB_TWIDDLE_A=1: always with pass A's stores
      if (R <= 128 && env_int("FFTGB_TWIDDLE_A") != 1 && !p->tw4_lo) {
        const int lgy = ilog2u(ny), bits = (lgy + 1) / 2;
        std::vector<float2> lo, hi;
        host_twiddles(lo, ny, 1LL << bits, 1);
        host_twiddles(hi, ny, (long long)ny >> bits, 1LL << bits);
        if (upload(&p->tw4_lo, lo) == FFTGB_OK && upload(&p->tw4_hi, hi) == FFTGB_OK) {
          p->tw4_bits = bits;
          b.in_mode = 1;
          b.tw4 = true;
          b.rows_log = ilog2u(nx);  // tw_shift
          p->twb = true;
        } else {
          cudaGetLastError();
        }
      }
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
      // out_mode 3: persistent, tiles copied in by TMA (one box per tile)
      const int pm = (pipe & 32) && fused_rz_tma_available((int)nz, R, X) ? 3 : 0;
      Pass b = {P_RZ, 0, 0, 0, pm, 0, 0, false, R, X};
      // 8 points per thread: twice the threads per tile, half the serial
      // chain of loads, butterflies and barriers in each (one-tile kernels,
      // each pass where it is built)
      if ((pipe & 8) && pa == 0 && fused_xy_available((int)nx, (int)nj, 8)) a.ept = 8;
      if ((pipe & 8) && pm == 0 && fused_rz_available((int)nz, R, X, 8)) b.ept = 8;
      p->passes.push_back(a);
      p->passes.push_back(b);
      // the y twiddle W_ny^(r*k1) goes with pass B's loads: R table reads
      // per tile instead of one per point in the issue-bound pass A
      // (FFTGB_TWIDDLE_A=1: with pass A's stores)
      p->twb = env_int("FFTGB_TWIDDLE_A") != 1;
      if (R > 1) p->inplace_ok = false;
      return;
    }
  }
}

// ------------------------------------------------------------ variants
// How a shape is split into kernel passes.  The choice is measured: the
// autotuner (fftgb_plan_autotune) times every candidate and records the
// fastest in the tuning cache; shapes never tuned use the defaults below,
// which come from measurements on GB300.
static std::string variant_str(const Variant &v) {
  char b[48];
  switch (v.kind) {
    case V_AXIS: return v.x == 8 ? "axis:b8" : "axis";
    case V_FUSED:
      if (v.pipe)
        snprintf(b, sizeof(b), "fused:%d:%d:p%d", v.nj, v.x, v.pipe);
      else
        snprintf(b, sizeof(b), "fused:%d:%d", v.nj, v.x);
      return b;
    case V_CLUSTER:
      if (!v.x) return "cluster";
      snprintf(b, sizeof(b), "cluster:%d", v.x);
      return b;
    case V_FOURSTEP: return "fourstep";
    case V_NONPOW2: return v.x ? ((v.pipe & 1) ? "mixed:simple" : "mixed") : "bluestein";
    default: return "default";
  }
}

static bool parse_variant(const std::string &s, Variant *v) {
  *v = Variant{V_DEFAULT, 0, 0};
  if (s == "axis") v->kind = V_AXIS;
  else if (s == "axis:b8") *v = Variant{V_AXIS, 0, 8};
  else if (s == "cluster") v->kind = V_CLUSTER;
  else if (sscanf(s.c_str(), "cluster:%d", &v->x) == 1) v->kind = V_CLUSTER;
  else if (s == "fourstep") v->kind = V_FOURSTEP;
  else if (s == "mixed") *v = Variant{V_NONPOW2, 0, 1};
  else if (s == "mixed:simple") *v = Variant{V_NONPOW2, 0, 1, 1};
  else if (s == "bluestein") *v = Variant{V_NONPOW2, 0, 0};
  else if (sscanf(s.c_str(), "fused:%d:%d", &v->nj, &v->x) == 2) {
    v->kind = V_FUSED;
    int pm = 0;
    // only the TMA bits remain (cache entries of removed forms run the one-tile kernels)
    if (sscanf(s.c_str(), "fused:%*d:%*d:p%d", &pm) == 1 && pm >= 0 && pm <= 63)
      v->pipe = pm & 56;
  }
  else return false;
  return true;
}

static std::string shape_key(unsigned nx, unsigned ny, unsigned nz,
                             unsigned batch, unsigned flags) {
  char key[96];
  snprintf(key, sizeof(key), "%u,%u,%u,%u,%u", nx, ny, nz, batch, flags);
  return key;
}

// Measured defaults (fused tile per cubic shape; 1D: the four-step's two
// 93 %-of-peak passes beat the cluster kernel on GB300).
// The first entry whose shape matches and whose min_batch <= batch wins.
// For one or two 256^3 grids the one-tile pass A of 32 rows (two CTAs per
// SM) with the TMA pass B in its radix-8 lane form (X = 4) leads: x 1
// 0.120 ms against 0.128 for the one-tile pair 32:8, x 2 0.217 against
// 0.221 for 64:8:p48.  From four grids on, both passes fed by TMA tensor
// copies with NJ = 64, X = 8 lead (pass B also storing by TMA): x 8 0.778
// ms against 0.791 for 32:4:p32 (pass A 0.372 against 0.407 ms, but pass B
// with 32-byte runs 0.416 against 0.367), 0.833 with the one-tile pass B
// (cp.async pass A 0.885, both passes cp.async 0.900, 32:8 0.889-0.909).  128^3 from four grids:
// the one-tile pass A with the TMA pass B (X = 16), x 4 0.0651 against
// 0.0668 ms, x 16 0.211 against 0.218, x 64 0.794 against 0.797 (x 1 a tie,
// 0.0284 against 0.0282).  The TMA pass A loses at 128^3 (x 16 0.235).
// 64^3: the one-tile pair with 8 points per thread leads at every batch
// (x 1 0.0083 against 0.0103 ms, x 16 0.0288 against 0.0349, x 64 0.109
// against 0.134; x 4 a tie).
struct FusedPref {
  unsigned nx, ny, nz, min_batch;
  int nj, x, pipe;
};
static const FusedPref kFusedPref[] = {
    {256, 256, 256, 4, 64, 8, 48}, {256, 256, 256, 1, 32, 4, 32},
    {128, 128, 128, 4, 64, 16, 32}, {128, 128, 128, 1, 64, 32, 0},
    {64, 64, 64, 1, 64, 32, 8},
};

static Variant choose_variant(unsigned nx, unsigned ny, unsigned nz,
                              unsigned batch, unsigned flags);

static int build_plan_v(fftgb_plan *out, int rank, unsigned nx, unsigned ny,
                        unsigned nz, unsigned batch, unsigned flags,
                        Variant var);

// Tuning cache file: a flat JSON object {"<shape key>": "<variant>", ...}.
static void tune_load(const std::string &path) {
  FILE *f = fopen(path.c_str(), "r");
  if (!f) return;
  std::string s;
  char buf[4096];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), f)) > 0) s.append(buf, n);
  fclose(f);
  // pairs of quoted strings separated by ':'
  size_t i = 0;
  while (true) {
    size_t a = s.find('"', i);
    if (a == std::string::npos) break;
    size_t b = s.find('"', a + 1);
    if (b == std::string::npos) break;
    size_t c = s.find('"', b + 1);
    if (c == std::string::npos) break;
    size_t d = s.find('"', c + 1);
    if (d == std::string::npos) break;
    const std::string key = s.substr(a + 1, b - a - 1);
    const std::string val = s.substr(c + 1, d - c - 1);
    Variant v;
    if (s.substr(b + 1, c - b - 1).find(':') != std::string::npos &&
        parse_variant(val, &v))
      g.tune[key] = val;
    i = d + 1;
  }
}

static void tune_save() {
  if (g.tune_path.empty()) return;
  FILE *f = fopen(g.tune_path.c_str(), "w");
  if (!f) return;
  fprintf(f, "{\n");
  size_t k = 0;
  for (const auto &kv : g.tune)
    fprintf(f, "  \"%s\": \"%s\"%s\n", kv.first.c_str(), kv.second.c_str(),
            ++k < g.tune.size() ? "," : "");
  fprintf(f, "}\n");
  fclose(f);
}

// Only an empty file or a JSON object is adopted as the tuning cache, so a
// path that names some other file is never overwritten.
static bool looks_like_tune_file(const char *path) {
  FILE *f = fopen(path, "r");
  if (!f) return false;
  int c;
  do {
    c = fgetc(f);
  } while (c == ' ' || c == '\n' || c == '\r' || c == '\t');
  fclose(f);
  return c == EOF || c == '{';
}

static void tune_init() {
  if (g.tune_loaded) return;
  g.tune_loaded = true;
  const char *e = getenv("FFTGB_TUNE_CACHE");
  if (e && *e) {
    g.tune_path = e;
    tune_load(g.tune_path);
  }
}

// Resolution order: environment overrides (FFTGB_NO_FUSED=1, FFTGB_FUSED_NJ
// / FFTGB_FUSED_X, FFTGB_CLUSTER=1, FFTGB_NO_CLUSTER=1), the tuning cache,
// the measured defaults, then the widest fused tile that fits.
static Variant choose_variant(unsigned nx, unsigned ny, unsigned nz,
                              unsigned batch, unsigned flags) {
  tune_init();
  if (ny == 1 && nz == 1) {
    if (env_int("FFTGB_CLUSTER") == 1)
      return Variant{V_CLUSTER, 0, env_int("FFTGB_CLUSTER_SIZE")};
    if (env_int("FFTGB_NO_CLUSTER") == 1) return Variant{V_FOURSTEP, 0, 0};
  } else {
    if (env_int("FFTGB_NO_FUSED") == 1) return Variant{V_AXIS, 0, 0};
    if (env_int("FFTGB_FUSED_NJ") || env_int("FFTGB_FUSED_X"))
      return Variant{V_FUSED, env_int("FFTGB_FUSED_NJ"), env_int("FFTGB_FUSED_X"),
                     env_int("FFTGB_FUSED_PIPE") & 63};
  }
  auto it = g.tune.find(shape_key(nx, ny, nz, batch, flags));
  Variant v;
  if (it != g.tune.end() && parse_variant(it->second, &v)) return v;
  if (ny == 1 && nz == 1) {
    // measured on GB300 against the four-step as a column pass and a row
    // pass (per forward): 32768 points, 8-CTA clusters lead up to about
    // 1024 transforms (x 512: 0.0940 against 0.0975 ms; x 64 0.0166 against
    // 0.0179) and the four-step above (x 2048: 0.336 against 0.343);
    // 65536 points, 16-CTA clusters for small batches (x 8: 0.0105 against
    // 0.0124 ms), the four-step from 32 on (x 32: 0.0185 against 0.0189;
    // x 64: 0.0328 against 0.0330; x 1024: 0.343 against 0.434)
    if (nx == 32768 && batch <= 1024 && cluster1d_available((int)nx, 8, nullptr, nullptr))
      return Variant{V_CLUSTER, 0, 8};
    if (nx == 65536 && batch <= 16 && cluster1d_available((int)nx, 16, nullptr, nullptr))
      return Variant{V_CLUSTER, 0, 16};
    return Variant{V_FOURSTEP, 0, 0};
  }
  // 3D grids with sides 16, 32, 64: one launch per direction on a 16-CTA
  // cluster holding the grid on chip.  It is the default up to 2^15 points
  // and a tuning choice above (FFTGB_CLUSTER=1 forces it, FFTGB_NO_CLUSTER=1
  // keeps the two-pass plans).  Measured on GB300 per forward transform:
  // 32^3 x 1 0.0063 against 0.0067 ms, 32^3 x 64 0.0209 against 0.0249,
  // 16^3 x 64 0.0063 against 0.0124; but 64^3 x 1 0.0267 against 0.0087 and
  // 64^3 x 64 0.224 against 0.130: one cluster spreads a grid over only 16
  // SMs, and a 64^3 grid's 16384 points per SM leave the kernel bound by
  // instruction issue, while the two-pass kernels spread it over 64-128 SMs.
  if (nz > 1 && env_int("FFTGB_NO_CLUSTER") != 1 &&
      cluster3d_available((int)nx, (int)ny, (int)nz) &&
      ((unsigned long long)nx * ny * nz <= 32768ULL || env_int("FFTGB_CLUSTER") == 1))
    return Variant{V_CLUSTER, 0, 0};
  for (const FusedPref &f : kFusedPref)
    if (f.nx == nx && f.ny == ny && f.nz == nz && batch >= f.min_batch)
      return Variant{V_FUSED, f.nj, f.x, f.pipe};
  if (nz == 1) {
    // 2D, measured on GB300: both plans make two passes, and up to 512 the
    // plain axis passes are as fast as any fused split (512^2 x 256: 0.408
    // against 0.413 ms; 256^2 x 1024: 0.347 against 0.368 ms); wider rows
    // gain from pass-A tiles of 8192 points, two CTAs per SM (1024^2 x 64:
    // 8 rows 0.391 ms, 16 rows 0.475, axis 0.489; 2048^2 x 16: 4 rows
    // 0.423, axis 0.514).  Wider rows over 128-512-point columns (the TMA
    // column pass) keep the axis passes on large batches: 1024 x 512 x 128
    // 0.369 against 0.398 ms, x 256 rows of 1024 0.356 against 0.377, 2048
    // x 256 x 128 0.369 against 0.396 (x 1 of 1024 x 512: fused 0.0105
    // against 0.0125)
    if (nx <= 512 && ny <= 512) return Variant{V_AXIS, 0, 0};
    if (ny >= 128 && ny <= 512 && nx <= 2048 &&
        (unsigned long long)nx * ny * batch >= (1ULL << 23))
      return Variant{V_AXIS, 0, 0};
    const unsigned nj = 8192 / nx;
    if (nj >= 2 && nj <= ny && fused_xy_available((int)nx, (int)nj))
      return Variant{V_FUSED, (int)nj, 0};
  }
  return Variant{V_FUSED, 0, 0};
}

static int build_plan(fftgb_plan *out, int rank, unsigned nx, unsigned ny,
                      unsigned nz, unsigned batch, unsigned flags) {
  return build_plan_v(out, rank, nx, ny, nz, batch, flags,
                      choose_variant(nx, ny, nz, batch, flags));
}

// In-place radix-2 FFT in FP64 (sign -1), n a power of two (host tables).
static void host_fft64(std::vector<double> &re, std::vector<double> &im) {
  const size_t n = re.size();
  for (size_t i = 1, j = 0; i < n; i++) {
    size_t bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      std::swap(re[i], re[j]);
      std::swap(im[i], im[j]);
    }
  }
  for (size_t len = 2; len <= n; len <<= 1) {
    const double a = -6.283185307179586476925286766559 / (double)len;
    for (size_t k = 0; k < len / 2; k++) {
      const double wr = cos(a * (double)k), wi = sin(a * (double)k);
      for (size_t b = 0; b < n; b += len) {
        const size_t p = b + k, q = p + len / 2;
        const double xr = re[q] * wr - im[q] * wi, xi = re[q] * wi + im[q] * wr;
        re[q] = re[p] - xr;
        im[q] = im[p] - xi;
        re[p] += xr;
        im[p] += xi;
      }
    }
  }
}

// Bluestein tables of axis length n: chirp w[m] = e^(-i pi m^2/n) (m^2 mod 2n
// in integers, the angle in FP64) and H = DFT_M(b) / M with b[m] = conj w[m]
// for |m| < n wrapped mod M.
static int blue_tables(unsigned n, int m_len, float2 **w_dev, float2 **h_dev) {
  std::vector<float2> w(n);
  std::vector<double> br(m_len, 0.0), bi(m_len, 0.0);
  const double pi = 3.14159265358979323846264338327950288;
  for (unsigned m = 0; m < n; m++) {
    const unsigned long long e = ((unsigned long long)m * m) % (2ULL * n);
    const double a = -pi * (double)e / (double)n;
    const double c = cos(a), sn = sin(a);
    w[m] = make_float2((float)c, (float)sn);
    br[m] = c;
    bi[m] = -sn;  // conj w
    if (m) {
      br[m_len - m] = c;
      bi[m_len - m] = -sn;
    }
  }
  host_fft64(br, bi);
  std::vector<float2> h(m_len);
  for (int k = 0; k < m_len; k++)
    h[k] = make_float2((float)(br[k] / m_len), (float)(bi[k] / m_len));
  int rc = upload(w_dev, w);
  if (!rc) rc = upload(h_dev, h);
  return rc;
}

// Twiddle table of the mixed-radix axis kernel: w[i] = e^(-2 pi i i/n) in
// FP64, rounded to FP32.
static int mix_table(unsigned n, float2 **w_dev) {
  std::vector<float2> w(n);
  const double pi = 3.14159265358979323846264338327950288;
  for (unsigned i = 0; i < n; i++) {
    const double a = -2.0 * pi * (double)i / (double)n;
    w[i] = make_float2((float)cos(a), (float)sin(a));
  }
  return upload(w_dev, w);
}

// A long 1D length n = 2^a 3^b 5^c (n > 4096) as n1 * n2 for the two four-step
// passes: both factors 16..4096, two-stage factorisations (the instantiated
// kernels) where possible, then the most balanced split.
static bool mix_fourstep_split(unsigned n, bool simple, unsigned *n1, unsigned *n2) {
  long long best = -1;
  for (unsigned a = 16; a <= 4096 && a <= n / 16; a++) {
    if (n % a) continue;
    const unsigned b = n / a;
    if (b < 16 || b > 4096) continue;
    int ra[MIX_MAXST], rb[MIX_MAXST];
    const int sa = mix_radices((int)a, ra, simple), sb = mix_radices((int)b, rb, simple);
    if (sa < 1 || sb < 1) continue;
    const int extra = (sa > 2 ? sa - 2 : 0) + (sb > 2 ? sb - 2 : 0);
    const long long imbalance = a > b ? (long long)a / b : (long long)b / a;
    const long long score = (long long)extra * 1000000 + imbalance * 1000 + (a < b ? 0 : 1);
    if (best < 0 || score < best) {
      best = score;
      *n1 = a;
      *n2 = b;
    }
  }
  return best >= 0;
}

// The four-step twiddles W_N^e of a long 1D transform as two levels:
// lo[e & 4095] = W_N^(e mod 4096), hi[e >> 12] = W_N^(4096 (e >> 12)), FP64.
static int fourstep_tables(unsigned N, float2 **lo_dev, float2 **hi_dev) {
  const double pi = 3.14159265358979323846264338327950288;
  std::vector<float2> lo(4096), hi(N / 4096 + 1);
  for (unsigned e = 0; e < 4096; e++) {
    const double a = -2.0 * pi * (double)e / (double)N;
    lo[e] = make_float2((float)cos(a), (float)sin(a));
  }
  for (size_t h = 0; h < hi.size(); h++) {
    const double a = -2.0 * pi * (double)(h * 4096 % N) / (double)N;
    hi[h] = make_float2((float)cos(a), (float)sin(a));
  }
  int rc = upload(lo_dev, lo);
  if (!rc) rc = upload(hi_dev, hi);
  return rc;
}

// Plans with an axis that is not a power of two: one pass per axis,
// power-of-two axes with k_rows / k_cols, lengths 2^a 3^b 5^c up to 8192 with
// the mixed-radix line kernel (kernels/fft_mix.cu), the others (length
// <= 2048) with the Bluestein line kernel (kernels/fft_blue.cu).
// FFTGB_NO_MIX=1 sends the smooth lengths to Bluestein too.
static int build_plan_blue(fftgb_plan *out, int rank, unsigned nx, unsigned ny,
                           unsigned nz, unsigned batch, unsigned flags, Variant var) {
  if ((flags & FFTGB_PREC_MASK) != FFTGB_PREC_FP32 || (flags & FFTGB_ORDER_BITREV)) {
    set_err("sizes that are not powers of two: FP32, natural order only");
    return FFTGB_EUNSUP;
  }
  const unsigned dims[3] = {nx, ny, nz};
  // the plan's variant: "mixed" (default), "mixed:simple" (radix 16, 8, 4, 2,
  // 5, 3 only) or "bluestein" (every axis that is not a power of two)
  const bool nonpow2_var = var.kind == V_NONPOW2;
  const bool no_mix = env_int("FFTGB_NO_MIX") == 1 || (nonpow2_var && var.x == 0);
  const bool simple = env_int("FFTGB_MIX_SIMPLE") == 1 || (nonpow2_var && (var.pipe & 1));
  for (int a = 0; a < 3; a++) {
    if (dims[a] == 0) {
      set_err("sizes must be at least 1");
      return FFTGB_EINVAL;
    }
    int rad[MIX_MAXST];
    const bool smooth = !no_mix && mix_radices((int)dims[a], rad, simple) > 0;
    unsigned f1, f2;
    const bool long1d = rank == 1 && a == 0 && !no_mix && !is_pow2(dims[a]) &&
                        dims[a] > 4096 && dims[a] <= (1u << 24) &&
                        mix_fourstep_split(dims[a], simple, &f1, &f2);
    if (!long1d && (is_pow2(dims[a]) ? dims[a] > 4096 : (dims[a] > 2048 && !smooth))) {
      set_err("axis length %u not supported (powers of two up to 4096, 2^a 3^b 5^c up "
              "to %d (1D: up to 2^24), others up to 2048)", dims[a], MIX_MAXN);
      return FFTGB_EUNSUP;
    }
  }
  unsigned fs1 = 0, fs2 = 0;  // 1D four-step split of a long length
  const bool fourstep = rank == 1 && !no_mix && !is_pow2(nx) && nx > 4096 &&
                        mix_fourstep_split(nx, simple, &fs1, &fs2);
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
  p->twb = false;
  p->tw4_lo = p->tw4_hi = nullptr;
  p->tw4_bits = 0;
  p->scratch = nullptr;
  p->natural_twin = nullptr;
  p->prof_max = 0;
  p->prof_count = 0;
  const long long total = (long long)p->points;
  long long inner = 1;
  if (fourstep) {
    // x[j1 + n1 j2]: the n2-point columns (stride n1) times W_N^(j1 k2), then
    // the n1-point rows stored transposed, X[k2 + n2 k1] (work buffer between)
    p->mix_nst[1] = mix_radices((int)fs2, p->mix_rad[1], simple);
    p->mix_nst[2] = mix_radices((int)fs1, p->mix_rad[2], simple);
    int rc = mix_table(fs2, &p->mix_w[1]);
    if (!rc) rc = mix_table(fs1, &p->mix_w[2]);
    if (!rc) rc = fourstep_tables(nx, &p->tw4_lo, &p->tw4_hi);
    if (rc) {
      plan_free(p);
      return rc;
    }
    p->tw4_bits = 12;
    Pass pa = {P_MIX, 0, total / fs2, (long long)fs1, 1, 0, 0, false, (int)fs2, 1};
    Pass pb = {P_MIX, 0, total / fs1, 1, 2, 0, 0, false, (int)fs1, 2};
    p->passes.push_back(pa);
    p->passes.push_back(pb);
    p->needs_work = true;
  }
  for (int a = 0; a < 3 && !fourstep; a++) {
    const unsigned n = dims[a];
    if (n > 1) {
      if (is_pow2(n)) {
        Pass ps = {a == 0 ? P_ROWS : P_COLS, ilog2u(n), total / n, a == 0 ? 0 : inner,
                   0, 0, 0, false, 0, 0};
        p->passes.push_back(ps);
      } else if (!no_mix && (p->mix_nst[a] = mix_radices((int)n, p->mix_rad[a], simple)) > 0) {
        const int rc = mix_table(n, &p->mix_w[a]);
        if (rc) {
          plan_free(p);
          return rc;
        }
        Pass ps = {P_MIX, 0, total / n, inner, 0, 0, 0, false, (int)n, a};
        p->passes.push_back(ps);
      } else {
        const int m = blue_length((int)n);
        const int rc = blue_tables(n, m, &p->blue_w[a], &p->blue_h[a]);
        if (rc) {
          plan_free(p);
          return rc;
        }
        Pass ps = {P_BLUE, ilog2u((unsigned)m), total / n, inner, 0, 0, 0, false, (int)n, a};
        p->passes.push_back(ps);
      }
    }
    inner *= n;
  }
  if (p->passes.empty()) {
    Pass c = {P_COPY, 0, total, 0, 0, 0, 0, false, 0, 0};
    p->passes.push_back(c);
  }
  bool any_blue = false;
  for (const Pass &ps : p->passes) any_blue = any_blue || ps.kind == P_BLUE;
  // "mixed": every non-power-of-two axis mixed-radix; "bluestein": some axis
  // takes Bluestein's algorithm
  p->variant = Variant{V_NONPOW2, 0, any_blue ? 0 : 1, (simple && !any_blue) ? 1 : 0};
  const int np = (int)p->passes.size();
  for (int i = 0; i < np; i++) {
    const Pass &ps = p->passes[(size_t)i];
    char nm[64];
    if (ps.kind == P_BLUE) {
      snprintf(nm, sizeof(nm), "k_blue<%d,n=%d>", 1 << ps.log_l, ps.aux0);
    } else if (ps.kind == P_MIX) {
      int w = snprintf(nm, sizeof(nm), "k_mix<n=%d,", ps.aux0);
      for (int q = 0; q < p->mix_nst[ps.aux1] && w < (int)sizeof(nm) - 12; q++)
        w += snprintf(nm + w, sizeof(nm) - (size_t)w, q ? "x%d" : "%d", p->mix_rad[ps.aux1][q]);
      // four-step passes: ",tw" the twiddled columns, ",tr" the transposed rows
      snprintf(nm + w, sizeof(nm) - (size_t)w, "%s>",
               ps.out_mode == 1 ? ",tw" : ps.out_mode == 2 ? ",tr" : "");
    }
    else if (ps.kind == P_COPY)
      snprintf(nm, sizeof(nm), "memcpy");
    else
      snprintf(nm, sizeof(nm), "%s<%d>", ps.kind == P_ROWS ? "k_rows" : "k_cols", 1 << ps.log_l);
    p->pass_names.push_back(nm);
  }
  *out = p;
  return FFTGB_OK;
}

// The y-blocked per-axis 3D plan applies: z-planes of 2 MiB or more, the y
// axis a TMA column pass (128, 256 or 512 points; nx a multiple of its tile
// width), rows of at most 4096 points.
static bool blocked_axes_ok(unsigned nx, unsigned ny, unsigned nz, long long total) {
  if (nz < 2 || nx > 4096 || ny < 128 || ny > 512 || nz > 4096) return false;
  if ((unsigned long long)nx * ny < (1ULL << 18)) return false;
  if (env_int("FFTGB_NO_COLS_TMA") == 1) return false;
  return cols_tma_supported(ilog2u(ny), total / ny, (long long)nx);
}

static int build_plan_v(fftgb_plan *out, int rank, unsigned nx, unsigned ny,
                        unsigned nz, unsigned batch, unsigned flags,
                        Variant var) {
  *out = nullptr;
  if (batch == 0 || nx == 0 || ny == 0 || nz == 0) {
    set_err("sizes and batch must be at least 1");
    return FFTGB_EINVAL;
  }
  if (!is_pow2(nx) || !is_pow2(ny) || !is_pow2(nz))
    return build_plan_blue(out, rank, nx, ny, nz, batch, flags, var);
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
  p->twb = false;
  p->tw4_lo = p->tw4_hi = nullptr;
  p->tw4_bits = 0;
  p->scratch = nullptr;
  p->natural_twin = nullptr;
  p->prof_max = 0;
  p->prof_count = 0;
  const long long total = (long long)p->points;
  const bool bitrev = (rank == 1) && (flags & FFTGB_ORDER_BITREV);
  // the tensor-core form is built on the per-axis (and four-step) passes
  const int tcm = tc_mode(flags);
  if (tcm) var = Variant{rank == 1 ? V_FOURSTEP : V_AXIS, 0, 0};

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
    if (var.kind == V_CLUSTER && cluster1d_available((int)nx, var.x, &cl1, &cl2)) {
      // one pass: the four-step transpose goes through distributed shared
      // memory of a thread-block cluster (kernels/fft1d_cluster.cu); the
      // pass's `inner` holds the cluster size
      int csz = var.x;
      if (!csz) cluster1d_sizes((int)nx, &csz, 1);
      // in_mode: the exchange form (0 remote loads, 1 bulk copies), the
      // measured default unless FFTGB_C1D_FORM names an available one
      const int forms = cluster1d_exchange_forms((int)nx, csz);
      const char *fe = getenv("FFTGB_C1D_FORM");
      int push = (forms & 4) ? 1 : 0;
      if (fe && *fe) {
        const int want = atoi(fe);
        if (want >= 0 && want <= 1 && (forms >> want) & 1) push = want;
      }
      Pass c = {P_C1D, 0, (long long)batch, csz, bitrev ? 1 : 0, push, 0, true, cl1,
                cl2};
      p->passes.push_back(c);
    } else if (!bitrev && !tcm && env_int("FFTGB_1D_COLS") != 1 &&
               rows_transposed_supported(lg1, lg2)) {
      // natural order as a column pass and a row pass: the columns (L2
      // points, stride L1) keep their layout and take the twiddle
      // W_N^(n1*k2) on their outputs (the TMA-fed column kernel), then each
      // row k2 is an L1-point FFT over n1 whose outputs k1 go to k2 + L2*k1,
      // staged in shared memory so that the stores are runs of whole rows.
      // 65536 x 1024 on GB300: 0.168 + 0.157 ms against 0.183 + 0.191 for
      // the transposed column store followed by a column pass with the
      // twiddle on its loads (FFTGB_1D_COLS=1 keeps that plan).  The row
      // pass cannot run in place, so the intermediate needs the work buffer.
      Pass a = {P_COLS, lg2, batch * L1, L1, 0, 0, 0, true};
      Pass b = {P_ROWS, lg1, batch * L2, 0, 4, 0, lg2, false};
      p->passes.push_back(a);
      p->passes.push_back(b);
      p->needs_work = true;
    } else {
      // natural order: the twiddle W_N^(n1*k2) goes with the loads of the
      // second pass (FFTGB_TWIDDLE_PASS1=1: with the stores of the first)
      const bool tw_first = bitrev || tcm || env_int("FFTGB_TWIDDLE_PASS1") == 1;
      Pass a = {P_COLS, lg2, batch * L1, L1, bitrev ? 0 : 1, 0, 0, tw_first};
      p->passes.push_back(a);
    }
    if (!p->passes.empty() && (p->passes[0].kind == P_C1D || p->passes.size() == 2)) {
      // done
    } else if (bitrev) {
      Pass b = {P_ROWS, lg1, batch * L2, 0, 2, 0, lg2, false};
      p->passes.push_back(b);
      p->needs_work = true;
    } else {
      const bool tw_first = tcm || env_int("FFTGB_TWIDDLE_PASS1") == 1;
      // in_mode 1: the four-step twiddle multiplies this pass's inputs
      Pass b = {P_COLS, lg1, batch * L2, L2, 0, tw_first ? 0 : 1, 0, !tw_first};
      p->passes.push_back(b);
    }
    p->inplace_ok = p->passes[0].kind == P_C1D;
  } else {
    if (nx > 4096 || ny > 4096 || nz > 4096) {
      plan_free(p);
      set_err("axis length above 4096 not supported for rank %d", rank);
      return FFTGB_EUNSUP;
    }
    if (var.kind == V_CLUSTER && rank == 3 &&
        cluster3d_available((int)nx, (int)ny, (int)nz)) {
      // one launch: the grid stays in one cluster's shared memory between
      // the axes; in place allowed (all loads precede the first store)
      Pass c = {P_C3D, 0, (long long)batch, 0, 0, 0, 0, false, 0, 0};
      p->passes.push_back(c);
    }
    if (var.kind == V_FUSED && rank >= 2) plan_fused(p, var.nj, var.x, var.pipe);
    // The per-axis 3D plan with its intermediate in the y-blocked layout
    // [b][ny/8][nz][8][nx] when a z-plane is 2 MiB or more: pass 1 (x)
    // writes whole rows there, pass 2 (z) is a column pass of stride 8*nx,
    // pass 3 (y) reads 8-row blocks by 5D tensor copies and writes the
    // natural layout.  No pass then reads or writes columns of a 2 MiB
    // stride, whose tiles touch one 2 MiB page per row: the z pass of 512^3
    // took 0.383 ms at that stride against 0.347 / 0.349 ms for the same
    // kernel at 256 KiB / 32 KiB strides.  The intermediate needs the plan's
    // work buffer (pass 1 remaps rows, pass 3 restores them).  Default for the
    // per-axis fallback (FFTGB_NO_BLK=1 keeps the natural layout); not for
    // plans of the host-buffer calls.
    if (p->passes.empty() && rank == 3 && !tcm &&
        ((var.kind == V_AXIS && var.x == 8) ||
         (var.kind == V_FUSED && env_int("FFTGB_NO_BLK") != 1 &&
          !(flags & FFTGB_FLAG_NATURAL_AXES))) &&
        blocked_axes_ok(nx, ny, nz, total)) {
      Pass a = {P_ROWS, ilog2u(nx), total / nx, 0, 3, 0, 0, false, ilog2u(ny), ilog2u(nz)};
      Pass b = {P_COLS, ilog2u(nz), total / nz, 8LL * nx, 0, 0, 0, false, 0, 0};
      Pass c = {P_COLS, ilog2u(ny), total / ny, (long long)nx, 0, 0, 0, false, 0, 0};
      c.blk = ilog2u(nz);
      p->passes.push_back(a);
      p->passes.push_back(b);
      p->passes.push_back(c);
      p->needs_work = true;
      p->inplace_ok = false;
      var = Variant{V_AXIS, 0, 8};
    }
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
  if (var.kind == V_CLUSTER && rank > 1 && p->passes[0].kind != P_C3D)
    var = Variant{V_AXIS, 0, 0};  // not expressible
  p->variant = var;
  // aux0 2: the persistent column pass whose tiles arrive by TMA tensor
  // copies into two alternating buffers, the default where it applies
  // (FFTGB_NO_COLS_TMA=1: the one-tile kernel).  Measured on GB300 against
  // the one-tile kernel: 512^3 1.080 against 1.168 ms (y and z passes 0.364
  // and 0.371 against 0.401 and 0.422), 512^2 x 256 0.367 against 0.385,
  // 256^2 x 1024 0.329 against 0.340, 256^3 x 8 per axis 0.964 against 1.007,
  // bit-reversed 1D 65536 x 1024 first pass (twiddled outputs) 0.197 against
  // 0.201.  Passes with the twiddle on their inputs stay with k_cols.
  const bool cols_tma = env_int("FFTGB_NO_COLS_TMA") != 1;
  for (Pass &ps : p->passes)
    if (!tcm && cols_tma && ps.kind == P_COLS && ps.aux0 == 0 && ps.out_mode == 0 &&
        ps.in_mode == 0 && cols_tma_supported(ps.log_l, ps.count, ps.inner))
      ps.aux0 = 2;
  if (tcm) {
    for (Pass &ps : p->passes)
      if ((ps.kind == P_ROWS || ps.kind == P_COLS) && tc_available(ps.log_l) &&
          ps.out_mode == 0 && ps.in_mode == 0 && !ps.tw4)
        ps.tc = tcm;
  }
  for (const Pass &ps : p->passes) {
    char nm[48];
    if (ps.tc)
      snprintf(nm, sizeof(nm), "%s<%d,%s>",
               ps.kind == P_ROWS ? "k_rows_tc" : "k_cols_tc", 1 << ps.log_l,
               ps.tc == 1 ? "f16" : "bf16");
    else if (ps.kind == P_COPY)
      snprintf(nm, sizeof(nm), "memcpy");
    else if (ps.kind == P_XY && ps.ept != 16)
      snprintf(nm, sizeof(nm), "k_xy<%u,%d,e%d>", p->n[0], ps.aux0, ps.ept);
    else if (ps.kind == P_XY)
      snprintf(nm, sizeof(nm), "%s<%u,%d>",
               ps.out_mode == 3 ? "k_xy_tma" : "k_xy",
               p->n[0], ps.aux0);
    else if (ps.kind == P_C1D)
      snprintf(nm, sizeof(nm), "%s<%d,%d,%lld>", ps.in_mode ? "k_1d_push" : "k_1d_cluster",
               ps.aux0, ps.aux1, ps.inner);
    else if (ps.kind == P_C3D)
      snprintf(nm, sizeof(nm), "k_3d_cluster<%u,%u,%u>", p->n[0], p->n[1], p->n[2]);
    else if (ps.kind == P_RZ && ps.ept != 16)
      snprintf(nm, sizeof(nm), "k_rz<%u,%d,%d,e%d>", p->n[2], ps.aux0, ps.aux1, ps.ept);
    else if (ps.kind == P_RZ)
      snprintf(nm, sizeof(nm), "%s<%u,%d,%d>",
               ps.out_mode == 3 ? "k_rz_tma" : "k_rz",
               p->n[2], ps.aux0, ps.aux1);
    else
      snprintf(nm, sizeof(nm), "%s<%d>",
               ps.kind == P_ROWS ? "k_rows" : ps.aux0 == 2 ? "k_cols_tma"
               : "k_cols",
               1 << ps.log_l);
    p->pass_names.push_back(nm);
  }
  *out = p;
  return FFTGB_OK;
}

// Launch the plan's passes: in -> [work ...] -> out.
// Launches one pass of plan p from src to dst on stream s (sc scales its
// outputs); i is the pass's index, for error messages.  pdl: the previous
// operation on s is the previous pass's kernel, so this pass may be launched
// as its programmatic dependent (kernels that support it wait in-kernel).
static int launch_pass(fftgb_plan p, const Pass &ps, int i, const float2 *src, float2 *dst,
                       int inverse, float sc, cudaStream_t s, bool pdl = false,
                       int filter = 0) {
  cudaError_t e = cudaSuccess;
  if (ps.kind == P_ROWS) {
    RowsArgs a;
    a.in = src;
    a.out = dst;
    a.nrows = ps.count;
    a.tw = axis_tw(ps.log_l);
    a.scale = sc;
    a.swap_io = inverse ? 1 : 0;
    a.in_mode = ps.in_mode;
    a.out_mode = ps.out_mode;
    a.rows_log = ps.rows_log;
    if (ps.out_mode == 3) {
      a.blk_lny = ps.aux0;
      a.blk_lnz = ps.aux1;
    }
    if (ps.tc) {
      a.tw = stage_tw(ps.log_l, 16);
      e = launch_rows_tc(ps.log_l, ps.tc, a, s);
    } else {
      e = launch_rows(ps.log_l, a, s, pdl);
    }
  } else if (ps.kind == P_COLS) {
    ColsArgs a;
    a.in = src;
    a.out = dst;
    a.ncols = ps.count;
    a.inner = ps.inner;
    a.tw = axis_tw(ps.log_l);
    a.tw4_lo = ps.tw4 ? p->tw4_lo : nullptr;
    a.tw4_hi = ps.tw4 ? p->tw4_hi : nullptr;
    a.tw4_bits = p->tw4_bits;
    a.scale = sc;
    a.swap_io = inverse ? 1 : 0;
    a.out_mode = ps.out_mode;
    a.tw_in = ps.in_mode == 1 ? 1 : 0;
    a.tw_shift = ps.rows_log;
    if (ps.tc) {
      a.tw = stage_tw(ps.log_l, 16);
      e = launch_cols_tc(ps.log_l, ps.tc, a, s);
    } else if (ps.blk >= 0) {
      // the y-blocked input is read by tensor copies only (no fallback)
      a.blk_lnz = ps.blk;
      e = launch_cols_tma(ps.log_l, a, s, pdl);
    } else if (ps.aux0 == 2) {
      e = launch_cols_tma(ps.log_l, a, s, pdl);
      if (e == cudaErrorMisalignedAddress || e == cudaErrorNotSupported)
        e = launch_cols(ps.log_l, a, s, pdl);  // same result
    } else {
      e = launch_cols(ps.log_l, a, s, pdl);
    }
  } else if (ps.kind == P_BLUE) {
    BlueArgs a;
    a.in = src;
    a.out = dst;
    a.nlines = ps.count;
    a.inner = ps.inner;
    a.n = ps.aux0;
    a.tw = axis_tw(ps.log_l);
    a.w = p->blue_w[ps.aux1];
    a.H = p->blue_h[ps.aux1];
    a.scale = sc;
    e = launch_blue(ps.log_l, inverse ? 1 : 0, a, s);
  } else if (ps.kind == P_MIX) {
    MixArgs a;
    a.in = src;
    a.out = dst;
    a.nlines = ps.count;
    a.inner = ps.inner;
    a.n = ps.aux0;
    a.nst = p->mix_nst[ps.aux1];
    for (int q = 0; q < MIX_MAXST; q++) a.rad[q] = p->mix_rad[ps.aux1][q];
    a.w = p->mix_w[ps.aux1];
    a.scale = sc;
    a.epi = ps.out_mode;
    if (ps.out_mode == 1) {
      a.tw_lo = p->tw4_lo;
      a.tw_hi = p->tw4_hi;
    } else if (ps.out_mode == 2) {
      a.ep_N = (long long)p->n[0];
      a.ep_n2 = a.ep_N / ps.aux0;
    }
    e = launch_mix(inverse ? 1 : 0, a, s);
  } else if (ps.kind == P_C3D) {
    C3dArgs a;
    a.in = src;
    a.out = dst;
    a.batch = ps.count;
    a.tw_x = tw_table(ilog2u(p->n[0]));
    a.tw_y = tw_table(ilog2u(p->n[1]));
    a.tw_z = tw_table(ilog2u(p->n[2]));
    a.scale = sc;
    a.swap_io = inverse ? 1 : 0;
    e = launch_cluster3d((int)p->n[0], (int)p->n[1], (int)p->n[2], a, s);
  } else if (ps.kind == P_C1D) {
    C1dArgs a;
    a.in = src;
    a.out = dst;
    a.count = ps.count;
    a.tw_a = stage_tw(ilog2u((unsigned)ps.aux1), 16);
    a.tw_b = stage_tw(ilog2u((unsigned)ps.aux0), 16);
    a.tw4_lo = p->tw4_lo;
    a.tw4_hi = p->tw4_hi;
    a.tw4_bits = p->tw4_bits;
    a.bitrev = ps.out_mode;
    a.scale = sc;
    a.swap_io = inverse ? 1 : 0;
    a.push = ps.in_mode;
    e = launch_cluster1d((int)p->n[0], (int)ps.inner, a, s);
  } else if (ps.kind == P_XY || ps.kind == P_RZ) {
    FusedArgs a;
    a.in = src;
    a.out = dst;
    a.nx = (int)p->n[0];
    a.ny = (int)p->n[1];
    a.nz = (int)p->n[2];
    a.batch = p->batch;
    a.tw_x = stage_tw(ilog2u(p->n[0]), ps.ept);
    a.tw_y = tw_table(ilog2u(p->n[1]));
    a.tw_z = p->n[2] > 1 ? stage_tw(ilog2u(p->n[2]), ps.ept) : nullptr;
    a.tw_j = ps.kind == P_XY ? stage_tw(ilog2u((unsigned)ps.aux0), ps.ept) : nullptr;
    a.scale = sc;
    a.swap_io = inverse ? 1 : 0;
    a.twb = p->twb ? 1 : 0;
    a.filter = filter;
    if (ps.kind == P_XY) {
      e = cudaErrorMisalignedAddress;
      if (ps.out_mode == 3) {
        e = launch_fused_xy_tma(ps.aux0, a, s, pdl);
        if (e == cudaErrorNotSupported) e = cudaErrorMisalignedAddress;
      }
      // buffers not 16-byte aligned: the one-tile-per-CTA kernel (same result)
      if (e == cudaErrorMisalignedAddress) e = launch_fused_xy(ps.aux0, a, s, pdl, ps.ept);
    } else {
      e = cudaErrorMisalignedAddress;
      if (ps.out_mode == 3) {
        e = launch_fused_rz_tma(ps.aux0, ps.aux1, a, s, pdl);
        if (e == cudaErrorNotSupported) e = cudaErrorMisalignedAddress;
      }
      // buffers not 16-byte aligned: the one-tile-per-CTA kernel (same result)
      if (e == cudaErrorMisalignedAddress)
        e = launch_fused_rz(ps.aux0, ps.aux1, a, s, pdl, ps.ept);
    }
  } else {
    if (sc != 1.0f) {
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
  return FFTGB_OK;
}

// Pass B of the fused 3D plans (the one-tile and TMA forms) multiplies its
// outputs by a spectral filter as it stores them.
static bool fuses_filter(const Pass &ps) {
  return ps.kind == P_RZ && (ps.out_mode == 0 || ps.out_mode == 3);
}

// `filter` (FFTGB_FILTER_*): the outputs are multiplied by that spectral
// filter, by the last pass when it can (fuses_filter), else by one more
// element-wise kernel after it.
static int run_passes(fftgb_plan p, const float2 *in, float2 *out, float2 *work,
                      int inverse, float scale, cudaStream_t s, int filter = 0) {
  const int np = (int)p->passes.size();
  cudaEvent_t *ev = nullptr;
  if (p->prof_count < p->prof_max) {
    ev = &p->prof_ev[(size_t)p->prof_count * (size_t)(np + 1)];
    p->prof_count++;
  }
  // passes after the first follow their predecessor's kernel directly on s
  // (no event in between unless profiling): programmatic dependent launches
  static const bool pdl_ok = env_int("FFTGB_NO_PDL") != 1;
  for (int i = 0; i < np; i++) {
    const Pass &ps = p->passes[(size_t)i];
    if (ev) cudaEventRecord(ev[i], s);
    const float2 *src = (i == 0) ? in : work;
    float2 *dst = (i == np - 1) ? out : work;
    const bool pdl = pdl_ok && i > 0 && !ev && p->passes[(size_t)i - 1].kind != P_COPY;
    const bool last = i == np - 1;
    const int rc = launch_pass(p, ps, i, src, dst, inverse, last ? scale : 1.0f, s, pdl,
                               last && fuses_filter(ps) ? filter : 0);
    if (rc) return rc;
  }
  if (filter && !fuses_filter(p->passes.back())) {
    const cudaError_t e = launch_filter(out, (long long)p->points, (int)p->n[0],
                                        (int)p->n[1], (int)p->n[2], filter, s);
    if (e != cudaSuccess) {
      set_err("filter launch failed: %s", cudaGetErrorString(e));
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
  int rc = build_plan(out, rank, nx, ny, nz, batch, flags | FFTGB_FLAG_NATURAL_AXES);
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

static int plan_check_status(fftgb_plan plan);

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

// Copies overlapped with compute, as the reference's buffer rotation does
// (api/src/fft3d.c:551-705): the batch is cut into chunks of `per_chunk`
// grids; chunk i is copied in on s_in, transformed on the compute stream once
// its copy has landed, and copied out on s_out once transformed, so copy-in
// of chunk i + 1, compute of chunk i and copy-out of chunk i - 1 overlap.
// wall_time: exec_t is the wall time of the whole call and the pcie fields
// stay 0 (the reference's fftfpgaf_c2c_3d_ddr_batch, fft3d.c:489, 861);
// otherwise exec_t, pcie_write_t and pcie_read_t are the sums of the
// chunks' kernel, copy-in and copy-out times (each timed on its own stream).
static int run_chunked(unsigned nx, unsigned ny, unsigned nz, unsigned batch,
                       unsigned per_chunk, unsigned flags, const float2 *inp,
                       float2 *out, bool inv, bool wall_time, fpga_t *t) {
  if (per_chunk == 0 || per_chunk > batch) per_chunk = batch;
  const unsigned nch = (batch + per_chunk - 1) / per_chunk;
  const unsigned rem = batch - (nch - 1) * per_chunk;
  fftgb_plan pf = nullptr, pr = nullptr;
  int rc = cached_plan(&pf, nx, ny, nz, per_chunk, flags);
  if (!rc && rem != per_chunk) rc = cached_plan(&pr, nx, ny, nz, rem, flags);
  if (rc) return rc;
  const size_t grid = (size_t)nx * ny * nz;
  rc = ensure_dev_buffers(grid * batch);
  if (rc) return rc;
  while (g.cev.size() < (size_t)nch * 6) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    g.cev.push_back(e);
  }
  const double t0 = now_ms();
  int status = FFTGB_OK;
  unsigned done = 0;  // chunks fully enqueued
  for (unsigned i = 0; i < nch && status == FFTGB_OK; i++) {
    fftgb_plan p = (i == nch - 1 && pr) ? pr : pf;
    const size_t off = grid * per_chunk * i;
    const size_t bytes = p->points * sizeof(float2);
    float2 *din = g.d_in + off, *dout = g.d_out + off;
    cudaEvent_t *e = &g.cev[(size_t)i * 6];
    if (cudaEventRecord(e[0], g.s_in) != cudaSuccess ||
        cudaMemcpyAsync(din, inp + off, bytes, cudaMemcpyHostToDevice, g.s_in) !=
            cudaSuccess ||
        cudaEventRecord(e[1], g.s_in) != cudaSuccess ||
        cudaStreamWaitEvent(g.stream, e[1], 0) != cudaSuccess ||
        cudaEventRecord(e[2], g.stream) != cudaSuccess) {
      set_err("pipelined copy-in failed");
      status = FFTGB_ECUDA;
      break;
    }
    status = run_passes(p, din, dout, p->needs_work ? din : dout, inv, 1.0f, g.stream);
    if (status) break;
    if (cudaEventRecord(e[3], g.stream) != cudaSuccess ||
        cudaStreamWaitEvent(g.s_out, e[3], 0) != cudaSuccess ||
        cudaEventRecord(e[4], g.s_out) != cudaSuccess ||
        cudaMemcpyAsync(out + off, dout, bytes, cudaMemcpyDeviceToHost, g.s_out) !=
            cudaSuccess ||
        cudaEventRecord(e[5], g.s_out) != cudaSuccess) {
      set_err("pipelined copy-out failed");
      status = FFTGB_ECUDA;
      break;
    }
    done = i + 1;
  }
  cudaError_t e1 = cudaStreamSynchronize(g.s_in);
  cudaError_t e2 = cudaStreamSynchronize(g.stream);
  cudaError_t e3 = cudaStreamSynchronize(g.s_out);
  if (wall_time) {
    t->exec_t = now_ms() - t0;
  } else {
    for (unsigned i = 0; i < done; i++) {
      const cudaEvent_t *e = &g.cev[(size_t)i * 6];
      t->pcie_write_t += ev_ms(e[0], e[1]);
      t->exec_t += ev_ms(e[2], e[3]);
      t->pcie_read_t += ev_ms(e[4], e[5]);
    }
  }
  if (status) return status;
  if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) {
    set_err("pipelined transform failed: %s",
            cudaGetErrorString(e2 != cudaSuccess ? e2 : (e1 ? e1 : e3)));
    return FFTGB_ECUDA;
  }
  // a bounded device wait that gave up leaves invalid results behind
  status = plan_check_status(pf);
  if (!status && pr) status = plan_check_status(pr);
  return status;
}

// One 3D grid on host buffers with the per-axis plan (x rows, y columns of
// stride nx, z columns of stride nx*ny), the copy-in overlapped with the
// kernels: the x and y passes work plane by plane, so each slab of planes is
// transformed as soon as its copy-in lands, while later slabs are still
// arriving; the z pass, which needs every plane, follows, then one
// contiguous copy-out.  (Streaming the z pass out in column blocks would
// need strided host copies, which run at 15-55 GB/s on this link against
// 193 GB/s contiguous.)  pcie_write_t and exec_t are the slabs' summed
// copy-in and kernel times (plus the z pass), pcie_read_t the copy-out.
// Returns FFTGB_EUNSUP (nothing run) when the plan or size does not qualify.
static int run_slabs(fftgb_plan p, const float2 *inp, float2 *out, bool inv, fpga_t *t) {
  const unsigned nx = p->n[0], ny = p->n[1], nz = p->n[2];
  const size_t plane = (size_t)nx * ny, total = plane * nz;
  if (p->rank != 3 || p->batch != 1 || p->needs_work || p->passes.size() != 3 ||
      total * sizeof(float2) < ((size_t)64 << 20))
    return FFTGB_EUNSUP;
  const Pass &px = p->passes[0], &py = p->passes[1], &pz = p->passes[2];
  if (px.kind != P_ROWS || px.in_mode || px.out_mode || px.tc || py.kind != P_COLS ||
      py.inner != (long long)nx || py.out_mode || py.in_mode || py.tw4 || py.tc || py.aux0 == 1 ||
      pz.kind != P_COLS || pz.inner != (long long)plane || pz.out_mode || pz.in_mode ||
      pz.tw4 || pz.tc || pz.aux0 == 1)
    return FFTGB_EUNSUP;
  const size_t plane_bytes = plane * sizeof(float2);
  unsigned S = (unsigned)(((size_t)32 << 20) / plane_bytes);  // planes per slab
  if (S < 1) S = 1;
  if (S > nz / 2) S = nz / 2;
  const unsigned nslab = (nz + S - 1) / S;
  int rc = ensure_dev_buffers(total);
  if (rc) return rc;
  while (g.cev.size() < (size_t)(nslab + 1) * 4) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    g.cev.push_back(e);
  }
  int status = FFTGB_OK;
  unsigned slabs_done = 0;
  for (unsigned k = 0; k < nslab && status == FFTGB_OK; k++) {
    const unsigned z0 = k * S, np = (z0 + S <= nz) ? S : nz - z0;
    const size_t off = plane * z0;
    cudaEvent_t *e = &g.cev[(size_t)k * 4];
    if (cudaEventRecord(e[0], g.s_in) != cudaSuccess ||
        cudaMemcpyAsync(g.d_in + off, inp + off, plane_bytes * np, cudaMemcpyHostToDevice,
                        g.s_in) != cudaSuccess ||
        cudaEventRecord(e[1], g.s_in) != cudaSuccess ||
        cudaStreamWaitEvent(g.stream, e[1], 0) != cudaSuccess ||
        cudaEventRecord(e[2], g.stream) != cudaSuccess) {
      set_err("slab copy-in failed");
      status = FFTGB_ECUDA;
      break;
    }
    Pass a = px, b = py;
    a.count = (long long)np * ny;
    b.count = (long long)np * nx;
    status = launch_pass(p, a, 0, g.d_in + off, g.d_out + off, inv, 1.0f, g.stream);
    if (!status) status = launch_pass(p, b, 1, g.d_out + off, g.d_out + off, inv, 1.0f, g.stream);
    if (!status && cudaEventRecord(e[3], g.stream) != cudaSuccess) {
      set_err("slab event record failed");
      status = FFTGB_ECUDA;
    }
    if (!status) slabs_done = k + 1;
  }
  bool z_done = false;
  if (status == FFTGB_OK) {
    cudaEvent_t *e = &g.cev[(size_t)nslab * 4];
    status = cudaEventRecord(e[0], g.stream) == cudaSuccess ? FFTGB_OK : FFTGB_ECUDA;
    if (status) set_err("event record failed");
    if (!status) status = launch_pass(p, pz, 2, g.d_out, g.d_out, inv, 1.0f, g.stream);
    if (!status) {
      if (cudaEventRecord(e[1], g.stream) != cudaSuccess ||
          cudaStreamWaitEvent(g.s_out, e[1], 0) != cudaSuccess ||
          cudaEventRecord(e[2], g.s_out) != cudaSuccess ||
          cudaMemcpyAsync(out, g.d_out, total * sizeof(float2), cudaMemcpyDeviceToHost,
                          g.s_out) != cudaSuccess ||
          cudaEventRecord(e[3], g.s_out) != cudaSuccess) {
        set_err("copy-out failed");
        status = FFTGB_ECUDA;
      } else {
        z_done = true;
      }
    }
  }
  cudaError_t e1 = cudaStreamSynchronize(g.s_in);
  cudaError_t e2 = cudaStreamSynchronize(g.stream);
  cudaError_t e3 = cudaStreamSynchronize(g.s_out);
  for (unsigned k = 0; k < slabs_done; k++) {
    const cudaEvent_t *e = &g.cev[(size_t)k * 4];
    t->pcie_write_t += ev_ms(e[0], e[1]);
    t->exec_t += ev_ms(e[2], e[3]);
  }
  if (z_done) {
    const cudaEvent_t *e = &g.cev[(size_t)nslab * 4];
    t->exec_t += ev_ms(e[0], e[1]);
    t->pcie_read_t += ev_ms(e[2], e[3]);
  }
  if (status) return status;
  if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) {
    set_err("slab pipeline failed: %s",
            cudaGetErrorString(e2 != cudaSuccess ? e2 : (e1 ? e1 : e3)));
    return FFTGB_ECUDA;
  }
  return FFTGB_OK;
}

// Grids per chunk of the copy pipeline of a host-buffer call, 0 when the call
// runs unchunked: only batches above 64 MiB are cut (smaller calls are
// latency-bound and gain nothing), into chunks of about 32 MiB, and only when
// the host buffers are the same or disjoint (a chunk's output may then land
// while later chunks' inputs are still being read).
static unsigned copy_chunk_grids(size_t grid_points, unsigned batch, const float2 *inp,
                                 const float2 *out) {
  const size_t grid_bytes = grid_points * sizeof(float2);
  const size_t total = grid_bytes * batch;
  if (batch < 2 || total < ((size_t)64 << 20)) return 0;
  const char *a = (const char *)inp, *b = (const char *)out;
  if (a != b && a < b + total && b < a + total) return 0;
  size_t per = ((size_t)32 << 20) / grid_bytes;
  if (per < 1) per = 1;
  if (per > batch / 2) per = batch / 2;
  return (unsigned)per;
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
  // the path doubles as the tuning cache when it is one (empty or JSON)
  tune_init();
  if (looks_like_tune_file(path)) {
    g.tune_path = path;
    tune_load(g.tune_path);
  }
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
  for (int e = 0; e < 2; e++) {
    if (g.tws[e]) cudaFree(g.tws[e]);
    g.tws[e] = nullptr;
  }
  g.tw = nullptr;
  for (int i = 0; i < 4; i++) {
    if (g.ev[i]) cudaEventDestroy(g.ev[i]);
    g.ev[i] = nullptr;
  }
  for (cudaEvent_t e : g.cev) cudaEventDestroy(e);
  g.cev.clear();
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
  const unsigned per =
      mode == FFTGB_RUN_COPY ? copy_chunk_grids((size_t)nx * ny * nz, batch, inp, out) : 0;
  if (mode == FFTGB_RUN_PIPELINE) {
    rc = run_chunked(nx, ny, nz, batch, 1, flags, inp, out, inv, true, &t);
  } else if (per) {
    rc = run_chunked(nx, ny, nz, batch, per, flags, inp, out, inv, false, &t);
  } else {
    fftgb_plan p = nullptr;
    rc = cached_plan(&p, nx, ny, nz, batch, flags);
    if (!rc && mode == FFTGB_RUN_COPY) {
      rc = run_slabs(p, inp, out, inv, &t);
      if (rc == FFTGB_EUNSUP) rc = run_copy(p, inp, out, inv, &t);
    } else if (!rc) {
      rc = (mode == FFTGB_RUN_SVM) ? run_svm(p, inp, out, inv, &t)
                                   : run_copy(p, inp, out, inv, &t);
    }
    // a bounded device wait that gave up leaves invalid results behind
    if (!rc) rc = plan_check_status(p);
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
  const unsigned prec = flags & FFTGB_PREC_MASK;
  if (prec != FFTGB_PREC_FP32 && prec != FFTGB_PREC_TC_FP16 &&
      prec != FFTGB_PREC_TC_BF16) {
    set_err("unknown precision mode 0x%x", prec);
    return FFTGB_EINVAL;
  }
  rc = build_plan(plan, rank, nx, ny, nz, batch, flags & ~FFTGB_FLAG_NATURAL_AXES);
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

extern "C" int fftgb_exec_filtered(fftgb_plan plan, const void *d_in, void *d_out,
                                   int inverse, float scale, int filter, void *stream) {
  int rc = check_io(plan, d_in, d_out);
  if (rc) return rc;
  if (filter != FFTGB_FILTER_POISSON || plan->rank != 3) {
    set_err("filter %d needs a 3D plan and a known filter", filter);
    return FFTGB_EINVAL;
  }
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  rc = ensure_device();
  if (rc) return rc;
  float2 *out = (float2 *)d_out;
  float2 *work = plan->needs_work ? plan->scratch : out;
  return run_passes(plan, (const float2 *)d_in, out, work, inverse, scale,
                    (cudaStream_t)stream, filter);
}

extern "C" int fftgb_exec_adjoint_filtered(fftgb_plan plan, const void *d_in, void *d_out,
                                           int inverse, float scale, int filter,
                                           void *stream) {
  // 3D plans are never bit-reversed: the adjoint of the forward (inverse)
  // transform is the unnormalised inverse (forward) with the same scale
  return fftgb_exec_filtered(plan, d_in, d_out, inverse ? 0 : 1, scale, filter, stream);
}

extern "C" int fftgb_residual_sq(const void *d_a, const void *d_b, void *d_r, size_t n,
                                 double *d_sum, void *stream) {
  if (!d_a || !d_b || !d_sum) {
    set_err("residual: NULL pointer");
    return FFTGB_EINVAL;
  }
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  int rc = ensure_device();
  if (rc) return rc;
  const cudaError_t e = launch_sq_residual((const float2 *)d_a, (const float2 *)d_b,
                                           (float2 *)d_r, (long long)n, d_sum,
                                           (cudaStream_t)stream);
  if (e != cudaSuccess) {
    set_err("residual launch failed: %s", cudaGetErrorString(e));
    return FFTGB_ECUDA;
  }
  return FFTGB_OK;
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
    a.tw = axis_tw(ilog2u(n));
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

// ------------------------------------------------------------ autotuner
extern "C" int fftgb_tune_cache(const char *path) {
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  tune_init();
  // the named cache replaces what is in memory (entries of an earlier cache
  // or of autotuner runs); none: untuned defaults, nothing recorded
  if (path == NULL || !*path) {
    g.tune_path.clear();
    g.tune.clear();
    return FFTGB_OK;
  }
  FILE *f = fopen(path, "a");
  if (!f) {
    set_err("cannot open tuning cache %s", path);
    return FFTGB_EINVAL;
  }
  fclose(f);
  if (!looks_like_tune_file(path)) {
    set_err("%s is not a tuning cache (JSON object)", path);
    return FFTGB_EINVAL;
  }
  g.tune_path = path;
  g.tune.clear();
  tune_load(g.tune_path);
  return FFTGB_OK;
}

static int time_variant(int rank, const fftgb_plan ref, Variant v,
                        const float2 *in, float2 *out, int reps, float *ms) {
  fftgb_plan q = nullptr;
  int rc = build_plan_v(&q, rank, ref->n[0], ref->n[1], ref->n[2], ref->batch,
                        ref->flags, v);
  if (rc) return rc;
  rc = ensure_scratch(q);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (!rc && (cudaEventCreate(&e0) != cudaSuccess ||
              cudaEventCreate(&e1) != cudaSuccess))
    rc = FFTGB_ECUDA;
  float2 *work = q->needs_work ? q->scratch : out;
  for (int i = 0; !rc && i < 2; i++)
    rc = run_passes(q, in, out, work, 0, 1.0f, g.stream);
  if (!rc) cudaEventRecord(e0, g.stream);
  for (int i = 0; !rc && i < reps; i++)
    rc = run_passes(q, in, out, work, i & 1, 1.0f, g.stream);
  if (!rc) {
    cudaEventRecord(e1, g.stream);
    if (cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(ms, e0, e1) != cudaSuccess)
      rc = FFTGB_ECUDA;
    else
      *ms /= (float)reps;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  // a variant that cannot run here is skipped, not fatal
  if (rc == FFTGB_ECUDA) cudaGetLastError();
  plan_free(q);
  return rc;
}

extern "C" int fftgb_plan_autotune(fftgb_plan plan, int reps, char *report,
                                   size_t report_len) {
  if (!plan) return FFTGB_EINVAL;
  if (reps < 1) reps = 5;
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  int rc = ensure_device();
  if (rc) return rc;
  const unsigned nx = plan->n[0], ny = plan->n[1], nz = plan->n[2];
  std::vector<Variant> cand;
  if (plan->variant.kind == V_NONPOW2) {
    // the composite and the simple radix sets, and Bluestein where every
    // axis that is not a power of two is at most 2048 long
    bool any_smooth = false, simple_differs = false, blue_ok = true;
    for (int a = 0; a < 3; a++) {
      const unsigned n = plan->n[a];
      if (is_pow2(n)) continue;
      int r1[MIX_MAXST], r2[MIX_MAXST];
      const int s1 = mix_radices((int)n, r1, false), s2 = mix_radices((int)n, r2, true);
      if (s1 > 0) any_smooth = true;
      if (s1 != s2) simple_differs = true;
      for (int q = 0; q < s1 && q < s2; q++) simple_differs = simple_differs || r1[q] != r2[q];
      if (n > 2048) blue_ok = false;
    }
    if (any_smooth) cand.push_back(Variant{V_NONPOW2, 0, 1});
    if (any_smooth && simple_differs) cand.push_back(Variant{V_NONPOW2, 0, 1, 1});
    if (blue_ok) cand.push_back(Variant{V_NONPOW2, 0, 0});
    if (cand.size() < 2) {
      if (report && report_len) snprintf(report, report_len, "single candidate");
      return FFTGB_OK;
    }
  } else if (plan->rank == 1) {
    if (nx > 4096) {
      cand.push_back(Variant{V_FOURSTEP, 0, 0});
      int cs[8];
      const int ncs = cluster1d_sizes((int)nx, cs, 8);
      for (int i = 0; i < ncs; i++) cand.push_back(Variant{V_CLUSTER, 0, cs[i]});
    }
  } else {
    cand.push_back(Variant{V_AXIS, 0, 0});
    if (plan->rank == 3 && !(plan->flags & FFTGB_FLAG_NATURAL_AXES) &&
        blocked_axes_ok(nx, ny, nz, (long long)plan->points))
      cand.push_back(Variant{V_AXIS, 0, 8});
    if (nz > 1 && cluster3d_available((int)nx, (int)ny, (int)nz))
      cand.push_back(Variant{V_CLUSTER, 0, 0});
    for (unsigned nj = nz == 1 ? 2 : 16; nj <= ny; nj <<= 1) {
      if ((unsigned long long)nj * nx > 16384ULL ||
          !fused_xy_available((int)nx, (int)nj))
        continue;
      const bool ta = fused_xy_tma_available((int)nx, (int)nj);
      if (nz == 1) {
        cand.push_back(Variant{V_FUSED, (int)nj, 0});
        if (ta) cand.push_back(Variant{V_FUSED, (int)nj, 0, 16});
        continue;
      }
      for (int X : {64, 32, 16, 8, 4})
        if ((unsigned)X <= nx && fused_rz_available((int)nz, (int)(ny / nj), X)) {
          const bool tb = fused_rz_tma_available((int)nz, (int)(ny / nj), X);
          // pass A: one-tile (0) or TMA-fed (16); pass B: one-tile (0) or TMA (32)
          for (int ma : {0, 16})
            for (int mb : {0, 32}) {
              if ((ma == 16 && !ta) || (mb == 32 && !tb)) continue;
              cand.push_back(Variant{V_FUSED, (int)nj, X, ma | mb});
            }
          // 8 points per thread in the one-tile passes that have it (with
          // pass B by TMA where that exists)
          const bool ea = fused_xy_available((int)nx, (int)nj, 8);
          const bool eb = fused_rz_available((int)nz, (int)(ny / nj), X, 8);
          if (ea || eb) cand.push_back(Variant{V_FUSED, (int)nj, X, 8});
          if (ea && tb) cand.push_back(Variant{V_FUSED, (int)nj, X, 8 | 32});
        }
    }
  }
  std::string rep;
  if (cand.size() < 2) {
    if (report && report_len) snprintf(report, report_len, "single candidate");
    return FFTGB_OK;
  }
  float2 *in = nullptr, *out = nullptr;
  const size_t bytes = plan->points * sizeof(float2);
  if (cudaMalloc((void **)&in, bytes) != cudaSuccess ||
      cudaMalloc((void **)&out, bytes) != cudaSuccess) {
    if (in) cudaFree(in);
    cudaGetLastError();
    set_err("autotune buffers (%zu bytes) could not be allocated", 2 * bytes);
    return FFTGB_ENOMEM;
  }
  cudaMemsetAsync(in, 0, bytes, g.stream);
  // one untimed sweep first: the first timed candidate must not pay for
  // first-touch of the buffers or clock ramp-up
  for (const Variant &v : cand) {
    float ms = 0.f;
    time_variant(plan->rank, plan, v, in, out, 1, &ms);
  }
  Variant best = plan->variant;
  float best_ms = -1.f;
  for (const Variant &v : cand) {
    float ms = 0.f;
    const int r = time_variant(plan->rank, plan, v, in, out, reps, &ms);
    char line[96];
    if (r == FFTGB_OK) {
      snprintf(line, sizeof(line), "%s=%.4f ", variant_str(v).c_str(), ms);
      if (best_ms < 0.f || ms < best_ms) {
        best_ms = ms;
        best = v;
      }
    } else {
      snprintf(line, sizeof(line), "%s=fail ", variant_str(v).c_str());
    }
    rep += line;
  }
  cudaFree(in);
  cudaFree(out);
  if (best_ms < 0.f) {
    set_err("no variant ran");
    return FFTGB_ECUDA;
  }
  // rebuild the plan with the winner and swap it in
  fftgb_plan q = nullptr;
  rc = build_plan_v(&q, plan->rank, nx, ny, nz, plan->batch, plan->flags, best);
  if (rc) return rc;
  std::swap(plan->passes, q->passes);
  std::swap(plan->pass_names, q->pass_names);
  std::swap(plan->tw4_lo, q->tw4_lo);
  std::swap(plan->tw4_hi, q->tw4_hi);
  std::swap(plan->tw4_bits, q->tw4_bits);
  std::swap(plan->needs_work, q->needs_work);
  std::swap(plan->inplace_ok, q->inplace_ok);
  std::swap(plan->twb, q->twb);
  std::swap(plan->variant, q->variant);
  for (int a = 0; a < 3; a++) {
    std::swap(plan->blue_w[a], q->blue_w[a]);
    std::swap(plan->blue_h[a], q->blue_h[a]);
    std::swap(plan->mix_w[a], q->mix_w[a]);
    std::swap(plan->mix_nst[a], q->mix_nst[a]);
    for (int k = 0; k < MIX_MAXST; k++) std::swap(plan->mix_rad[a][k], q->mix_rad[a][k]);
  }
  plan_free(q);
  rc = ensure_scratch(plan);
  if (rc) return rc;
  g.tune[shape_key(nx, ny, nz, plan->batch, plan->flags)] = variant_str(best);
  tune_save();
  rep += "-> " + variant_str(best);
  if (report && report_len) snprintf(report, report_len, "%s", rep.c_str());
  return FFTGB_OK;
}

// Reads (and clears) the status words of the bounded device-side waits that
// the plan's kernels use; FFTGB_ETIMEOUT when one of them gave up.
static int plan_check_status(fftgb_plan plan) {
  if (plan->passes.empty()) return FFTGB_OK;
  if (plan->passes[0].kind == P_C1D && plan->passes[0].in_mode == 1) {
    const int st = cluster1d_status_and_clear();
    if (st < 0) return FFTGB_ECUDA;
    if (st) {
      set_err("a cluster bulk-copy exchange wait gave up");
      return FFTGB_ETIMEOUT;
    }
  }
  for (const Pass &ps : plan->passes) {
    if (ps.kind != P_COLS || ps.aux0 != 2) continue;
    const int st = cols_tma_status_and_clear();
    if (st < 0) return FFTGB_ECUDA;
    if (st) {
      set_err("a TMA column-tile completion wait gave up");
      return FFTGB_ETIMEOUT;
    }
    break;
  }
  for (const Pass &ps : plan->passes) {
    if ((ps.kind != P_XY && ps.kind != P_RZ) || ps.out_mode != 3) continue;
    const int st = fused_tma_status_and_clear();
    if (st < 0) return FFTGB_ECUDA;
    if (st) {
      set_err("a TMA tile-copy completion wait gave up");
      return FFTGB_ETIMEOUT;
    }
    break;
  }
  for (const Pass &ps : plan->passes) {
    if (!ps.tc) continue;
    const int st = tc_status_and_clear();
    if (st < 0) return FFTGB_ECUDA;
    if (st) {
      set_err("a tensor-core MMA completion wait gave up");
      return FFTGB_ETIMEOUT;
    }
    break;
  }
  return FFTGB_OK;
}

extern "C" int fftgb_debug_expire_wait(int family, unsigned polls) {
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  if (ensure_device() != FFTGB_OK) return FFTGB_ENODEV;
  if (polls > (1u << 20)) {
    set_err("polls above 2^20");
    return FFTGB_EINVAL;
  }
  cudaError_t e;
  switch (family) {
    case FFTGB_WAIT_COLS_TMA: e = cols_tma_expire_wait(polls); break;
    case FFTGB_WAIT_FUSED_TMA: e = fused_tma_expire_wait(polls); break;
    case FFTGB_WAIT_CLUSTER_1D: e = cluster1d_expire_wait(polls); break;
    case FFTGB_WAIT_TENSOR_CORE: e = tc_expire_wait(polls); break;
    default: set_err("unknown wait family %d", family); return FFTGB_EINVAL;
  }
  if (e != cudaSuccess) {
    set_err("expire-wait launch: %s", cudaGetErrorString(e));
    return FFTGB_ECUDA;
  }
  return FFTGB_OK;
}

extern "C" int fftgb_plan_status(fftgb_plan plan) {
  if (!plan) return FFTGB_EINVAL;
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  return plan_check_status(plan);
}

extern "C" const char *fftgb_plan_variant(fftgb_plan plan) {
  static thread_local std::string s;
  s = plan ? variant_str(plan->variant) : "";
  return s.c_str();
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

// Hooks for the ragged-batch planner (shim/ragged.cu).
namespace fftgb {
int internal_ensure_device(int *device) {
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  const int rc = ensure_device();
  if (!rc && device) *device = g.device;
  return rc;
}
const float2 *internal_axis_tw(int log_l) { return axis_tw(log_l); }
// Changes whenever fpga_final released the shared tables and they were
// created again: launch arguments captured before hold stale pointers.
unsigned internal_device_generation() {
  std::lock_guard<std::recursive_mutex> lk(g.mu);
  return g.generation;
}
const float2 *internal_stage_tw16(int log_l) { return stage_tw(log_l, 16); }
const float2 *internal_w_table(int log_l) { return tw_table(log_l); }
void internal_set_err(const char *msg) { set_err("%s", msg); }
}  // namespace fftgb

extern "C" const char *fftgb_last_error(void) { return g_errbuf; }

extern "C" const char *fftgb_version(void) { return "fftgb 0.1 (sm_103a)"; }
