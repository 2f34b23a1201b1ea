// noalloc.cu - fftgb_c2c_1d_noalloc: the bit-reversed 1D transform of
// fftfpgaf_c2c_1d on caller-owned device buffers, without allocating.
//
// Who needs it: callers that cannot call cudaMalloc.  Examples are
// applications whose device memory is owned entirely by their own pool
// allocator (a framework that reserves HBM at start-up and hands out slices),
// and latency-critical callers that must not allocate on the hot path
// because cudaMalloc can synchronise the whole device.  The regular plans
// (fftgb_plan_1d with FFTGB_ORDER_BITREV) allocate a plan scratch buffer and
// twiddle tables; this entry point uses file-scope device arrays instead.
//
// Memory it holds: every GPU that loads the library keeps the arrays below
// (8 MiB of scratch plus about 120 KiB of twiddle tables) until the process
// exits.  The first call on a device does the set-up for that device (symbol
// addresses, twiddle upload, kernel attributes); make that first call before
// any stream capture.  All calls share the one scratch array: calls whose
// work overlaps on the GPU (different streams, no ordering) race on it.
// The scratch is always fully written before it is read, so nothing has to
// be cleared between calls.  A cudaDeviceReset after the first call on a
// device is not supported: it reloads the module with zeroed twiddle arrays
// while this file still counts the device as set up (the tables are not
// uploaded again), so later calls on that device would be wrong.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>

#include <mutex>
#include <vector>

#include "fftfpga_ext.h"
#include "../kernels/fft_core.cuh"
#include "../kernels/fft_pass.cuh"
#include "tables.h"

using namespace fftgb;

// Largest transform length, and scratch capacity in complex points.
#define NA_MAX_LOG 20
#define NA_SCRATCH_POINTS (1u << NA_MAX_LOG)
static_assert(NA_SCRATCH_POINTS == FFTGB_NOALLOC_MAX_N,
              "the scratch array holds exactly the documented public limit");
// Stockham stage tables of the per-axis kernels for L = 2..4096, back to back
// (offsets in NaDevice::tw_off).
#define NA_TW_POINTS 9184
// Four-step tables for N = 2^13 .. 2^20: lo (2^ceil(lg/2)) then hi
// (2^floor(lg/2)) entries per size, back to back.
#define NA_TW4_POINTS 6720

static __device__ __align__(256) float2 g_na_scratch[NA_SCRATCH_POINTS];
static __device__ __align__(256) float2 g_na_tw[NA_TW_POINTS];
static __device__ __align__(256) float2 g_na_tw4[NA_TW4_POINTS];

namespace {
struct NaDevice {
  bool ready = false;
  float2 *scratch = nullptr;
  float2 *tw = nullptr;
  int tw_off[13] = {};
  float2 *tw4 = nullptr;
};
constexpr int kMaxDevices = 64;
NaDevice g_na[kMaxDevices];
std::mutex g_na_mu;
thread_local char g_na_err[256];

int na_fail(int code, const char *msg, cudaError_t e = cudaSuccess) {
  snprintf(g_na_err, sizeof(g_na_err), "fftgb_c2c_1d_noalloc: %s%s%s", msg,
           e != cudaSuccess ? ": " : "",
           e != cudaSuccess ? cudaGetErrorString(e) : "");
  return code;
}

void na_twiddles(std::vector<float2> &out, long long n, long long count,
                 long long step) {
  for (long long i = 0; i < count; i++) {
    const long long m = (i * step) % n;
    double s, c;
    sincos(-2.0 * M_PI * ((double)m / (double)n), &s, &c);
    float2 w;
    w.x = (float)c;
    w.y = (float)s;
    out.push_back(w);
  }
}

int na_tw4_offset(int lg) {
  int off = 0;
  for (int l = 13; l < lg; l++) off += (1 << ((l + 1) / 2)) + (1 << (l / 2));
  return off;
}

// Once per device, with that device current: resolve the device addresses of
// the file-scope arrays (the host-side symbols are not device addresses),
// upload the twiddle tables and set the kernels' shared-memory limits.
int na_setup(int dev) {
  NaDevice &d = g_na[dev];
  if (d.ready) return FFTGB_OK;
  cudaError_t e = cudaGetSymbolAddress((void **)&d.scratch, g_na_scratch);
  if (e != cudaSuccess) return na_fail(FFTGB_ECUDA, "scratch address", e);
  e = cudaGetSymbolAddress((void **)&d.tw, g_na_tw);
  if (e != cudaSuccess) return na_fail(FFTGB_ECUDA, "twiddle address", e);
  e = cudaGetSymbolAddress((void **)&d.tw4, g_na_tw4);
  if (e != cudaSuccess) return na_fail(FFTGB_ECUDA, "twiddle address", e);
  std::vector<float2> tw, tw4;
  for (int l = 1; l <= 12; l++) {
    d.tw_off[l] = (int)tw.size();
    stage_table(tw, 1 << l, default_e(1 << l));
  }
  for (int lg = 13; lg <= NA_MAX_LOG; lg++) {
    const int bits = (lg + 1) / 2;
    na_twiddles(tw4, 1LL << lg, 1LL << bits, 1);
    na_twiddles(tw4, 1LL << lg, 1LL << (lg - bits), 1LL << bits);
  }
  if (tw.size() != NA_TW_POINTS || tw4.size() != NA_TW4_POINTS)
    return na_fail(FFTGB_ECUDA, "twiddle table size mismatch");
  e = cudaMemcpyToSymbol(g_na_tw, tw.data(), tw.size() * sizeof(float2));
  if (e != cudaSuccess) return na_fail(FFTGB_ECUDA, "twiddle upload", e);
  e = cudaMemcpyToSymbol(g_na_tw4, tw4.data(), tw4.size() * sizeof(float2));
  if (e != cudaSuccess) return na_fail(FFTGB_ECUDA, "twiddle upload", e);
  e = pass_kernels_set_attributes_current_device();
  if (e != cudaSuccess) return na_fail(FFTGB_ECUDA, "kernel attributes", e);
  d.ready = true;
  return FFTGB_OK;
}
}  // namespace

extern "C" int fftgb_c2c_1d_noalloc(unsigned n, unsigned batch,
                                    const void *d_in, void *d_out, int inverse,
                                    void *stream) {
  if (d_in == NULL || d_out == NULL || batch == 0 || n < 2 || (n & (n - 1)))
    return na_fail(FFTGB_EINVAL, "bad argument (NULL buffer, batch 0, or n "
                                 "not a power of two >= 2)");
  if (n > NA_SCRATCH_POINTS)
    return na_fail(FFTGB_EUNSUP, "n above the 2^20-point scratch limit");
  const size_t bytes = (size_t)n * batch * sizeof(float2);
  const char *a = (const char *)d_in, *b = (const char *)d_out;
  if (a < b + bytes && b < a + bytes)
    return na_fail(FFTGB_EINVAL, "input and output overlap");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return na_fail(FFTGB_ENODEV, "no current CUDA device", e);
  NaDevice d;
  {
    std::lock_guard<std::mutex> lk(g_na_mu);
    const int rc = na_setup(dev);
    if (rc) return rc;
    d = g_na[dev];
  }
  cudaStream_t s = (cudaStream_t)stream;
  int lg = 0;
  while ((1u << lg) < n) lg++;
  const float2 *in = (const float2 *)d_in;
  float2 *out = (float2 *)d_out;

  if (n <= 4096) {
    // one pass, no scratch: bit-reversed store within each row
    RowsArgs r;
    r.in = in;
    r.out = out;
    r.nrows = batch;
    r.tw = d.tw + d.tw_off[lg];
    r.scale = 1.0f;
    r.swap_io = inverse ? 1 : 0;
    r.in_mode = 0;
    r.out_mode = 1;
    r.rows_log = 0;
    e = launch_rows_on(lg, r, s);
    if (e != cudaSuccess) return na_fail(FFTGB_ECUDA, "launch", e);
    return FFTGB_OK;
  }

  // four-step through the file-scope scratch, in rounds of at most
  // NA_SCRATCH_POINTS points
  const int lg2 = lg / 2, lg1 = lg - lg2;
  const long long L1 = 1LL << lg1, L2 = 1LL << lg2;
  const int bits = (lg + 1) / 2;
  const float2 *lo = d.tw4 + na_tw4_offset(lg);
  const float2 *hi = lo + (1 << bits);
  const unsigned per_round = NA_SCRATCH_POINTS / n;
  for (unsigned b0 = 0; b0 < batch; b0 += per_round) {
    const unsigned nb = (batch - b0 < per_round) ? (batch - b0) : per_round;
    ColsArgs c;
    c.in = in + (size_t)b0 * n;
    c.out = d.scratch;
    c.ncols = (long long)nb * L1;
    c.inner = L1;
    c.tw = d.tw + d.tw_off[lg2];
    c.tw4_lo = lo;
    c.tw4_hi = hi;
    c.tw4_bits = bits;
    c.scale = 1.0f;
    c.swap_io = inverse ? 1 : 0;
    c.out_mode = 0;
    e = launch_cols_on(lg2, c, s);
    if (e != cudaSuccess) return na_fail(FFTGB_ECUDA, "launch", e);
    RowsArgs r;
    r.in = d.scratch;
    r.out = out + (size_t)b0 * n;
    r.nrows = (long long)nb * L2;
    r.tw = d.tw + d.tw_off[lg1];
    r.scale = 1.0f;
    r.swap_io = inverse ? 1 : 0;
    r.in_mode = 0;
    r.out_mode = 2;
    r.rows_log = lg2;
    e = launch_rows_on(lg1, r, s);
    if (e != cudaSuccess) return na_fail(FFTGB_ECUDA, "launch", e);
  }
  return FFTGB_OK;
}

extern "C" const char *fftgb_noalloc_last_error(void) { return g_na_err; }
