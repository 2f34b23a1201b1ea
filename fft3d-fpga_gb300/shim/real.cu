// real.cu - real-data plans: R2C (real grid -> half spectrum) and C2R
// (half spectrum -> real grid, unnormalised), 1D/2D/3D, batched.  No
// counterpart in the reference (it has complex transforms only); the layout
// is the usual half-spectrum one: grid [batch][nz][ny][nx] of reals <->
// [batch][nz][ny][nx/2 + 1] complex, x fastest.
//
// R2C: the x pass (kernels/fft_real.cu) reads the real rows and writes the
// half-spectrum rows to the output, then the y and z column passes run in
// place there.  C2R: the z and y passes run on a plan-owned half-spectrum
// scratch buffer (the input is not modified), then the x pass writes the
// real rows.
//
// Lengths that are not powers of two (2^a 3^b 5^c; nx even with nx/2 of that
// form): the y and z passes are the mixed-radix axis kernel
// (kernels/fft_mix.cu) over the half-spectrum columns, and the x pass is its
// real-data form (kernels/fft_mix_real.cu) over the real rows packed as nx/2
// complex points, the split into (C2R: combination from) the M + 1 spectrum
// values fused into the same pass.
#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>

#include <vector>

#include "fftfpga_ext.h"
#include "../kernels/fft_mix.cuh"
#include "../kernels/fft_pass.cuh"
#include "../kernels/fft_real.cuh"

namespace fftgb {
int internal_ensure_device(int *device);
const float2 *internal_axis_tw(int log_l);
void internal_set_err(const char *msg);
}  // namespace fftgb

using namespace fftgb;

// One axis of a real-data plan taken by the mixed-radix kernel.
struct RealMixAxis {
  int n = 0;                // 0: not mixed-radix (power of two or unused)
  int nst = 0;
  int rad[MIX_MAXST] = {};
  float2 *w = nullptr;      // W_n^i, i < n
};

struct fftgb_rplan_s {
  int rank;
  unsigned nx, ny, nz, batch;
  size_t real_points, spec_points;
  float2 *wn;       // W_nx^k, k = 0..nx/2
  float2 *scratch;  // C2R with y or z passes: half-spectrum work buffer
  RealMixAxis mx, my, mz;  // x: the nx/2-point packed rows; y; z
};

static int ilog2(unsigned v) {
  int r = 0;
  while ((1u << r) < v) r++;
  return r;
}

static bool pow2(unsigned v) { return v && !(v & (v - 1)); }

// A mixed-radix axis of length n (not a power of two): its radices and W_n
// table (FP64, rounded to FP32).  Returns false on an allocation failure.
static bool mix_axis(RealMixAxis *ax, unsigned n) {
  ax->n = (int)n;
  const char *e = getenv("FFTGB_MIX_SIMPLE");
  ax->nst = mix_radices((int)n, ax->rad, e && atoi(e) == 1);
  std::vector<float2> w(n);
  for (unsigned i = 0; i < n; i++) {
    const double a = -6.283185307179586476925286766559 * (double)i / (double)n;
    w[i] = make_float2((float)cos(a), (float)sin(a));
  }
  return cudaMalloc((void **)&ax->w, n * sizeof(float2)) == cudaSuccess &&
         cudaMemcpy(ax->w, w.data(), n * sizeof(float2), cudaMemcpyHostToDevice) ==
             cudaSuccess;
}

// An axis length the real plans take: a power of two up to pow2_max, or
// 2^a 3^b 5^c up to the mixed-radix limit.
static bool axis_ok(unsigned n, unsigned pow2_max) {
  if (pow2(n)) return n <= pow2_max;
  int rad[MIX_MAXST];
  return mix_radices((int)n, rad) > 0;
}

// the mixed-radix pass over lines of n points ([outer][n][inner] layout)
static cudaError_t mix_pass(const RealMixAxis &ax, const float2 *in, float2 *out,
                            long long nlines, long long inner, int inverse, float scale,
                            cudaStream_t s) {
  MixArgs a;
  a.in = in;
  a.out = out;
  a.nlines = nlines;
  a.inner = inner;
  a.n = ax.n;
  a.nst = ax.nst;
  for (int q = 0; q < MIX_MAXST; q++) a.rad[q] = ax.rad[q];
  a.w = ax.w;
  a.scale = scale;
  return launch_mix(inverse, a, s);
}

// the x pass of the real-data plans with a mixed-radix nx/2 (c2r = 0: R2C)
static cudaError_t mix_real_pass(const RealMixAxis &ax, const float2 *wn, const float2 *in,
                                 float2 *out, long long nrows, int c2r, float scale,
                                 cudaStream_t s) {
  MixArgs a;
  a.in = in;
  a.out = out;
  a.nlines = nrows;
  a.inner = 1;
  a.n = ax.n;
  a.nst = ax.nst;
  for (int q = 0; q < MIX_MAXST; q++) a.rad[q] = ax.rad[q];
  a.w = ax.w;
  a.wn = wn;
  a.scale = scale;
  return launch_mix_real(c2r, a, s);
}

extern "C" int fftgb_plan_r2c(fftgb_rplan *plan, int rank, unsigned nx, unsigned ny,
                              unsigned nz, unsigned batch) {
  if (!plan) return FFTGB_EINVAL;
  *plan = NULL;
  if (rank < 1 || rank > 3 || batch == 0 || ny == 0 || nz == 0 || (rank < 2 && ny != 1) ||
      (rank < 3 && nz != 1)) {
    internal_set_err("r2c plan: rank 1-3, unused sizes 1, batch > 0");
    return FFTGB_EINVAL;
  }
  if (nx < 4 || nx > 8192 || (nx & 1) || !axis_ok(nx / 2, 4096) ||
      (ny > 1 && !axis_ok(ny, 4096)) || (nz > 1 && !axis_ok(nz, 4096))) {
    internal_set_err("r2c plan: nx even, 4..8192, with nx/2 a power of two or 2^a 3^b 5^c; "
                     "ny, nz powers of two up to 4096 or 2^a 3^b 5^c up to 8192");
    return FFTGB_EUNSUP;
  }
  int device = 0;
  int rc = internal_ensure_device(&device);
  if (rc) return rc;
  if (real_kernels_init() != cudaSuccess) {
    internal_set_err("real-data kernels could not be initialised");
    return FFTGB_ECUDA;
  }
  fftgb_rplan p = new fftgb_rplan_s();
  p->rank = rank;
  p->nx = nx;
  p->ny = ny;
  p->nz = nz;
  p->batch = batch;
  p->real_points = (size_t)nx * ny * nz * batch;
  p->spec_points = (size_t)(nx / 2 + 1) * ny * nz * batch;
  p->wn = NULL;
  p->scratch = NULL;
  const unsigned m = nx / 2;
  std::vector<float2> w(m + 1);
  for (unsigned k = 0; k <= m; k++) {
    const double a = -6.283185307179586476925286766559 * (double)k / (double)nx;
    w[k] = make_float2((float)cos(a), (float)sin(a));
  }
  bool okay = cudaMalloc((void **)&p->wn, w.size() * sizeof(float2)) == cudaSuccess &&
              cudaMemcpy(p->wn, w.data(), w.size() * sizeof(float2),
                         cudaMemcpyHostToDevice) == cudaSuccess;
  if (okay && (ny > 1 || nz > 1))
    okay = cudaMalloc((void **)&p->scratch, p->spec_points * sizeof(float2)) == cudaSuccess;
  if (okay && !pow2(m)) okay = mix_axis(&p->mx, m);
  if (okay && ny > 1 && !pow2(ny)) okay = mix_axis(&p->my, ny);
  if (okay && nz > 1 && !pow2(nz)) okay = mix_axis(&p->mz, nz);
  if (!okay) {
    cudaGetLastError();
    fftgb_rplan_destroy(p);
    internal_set_err("r2c plan allocation failed");
    return FFTGB_ENOMEM;
  }
  *plan = p;
  return FFTGB_OK;
}

extern "C" void fftgb_rplan_destroy(fftgb_rplan p) {
  if (!p) return;
  if (p->wn) cudaFree(p->wn);
  if (p->scratch) cudaFree(p->scratch);
  for (RealMixAxis *ax : {&p->mx, &p->my, &p->mz})
    if (ax->w) cudaFree(ax->w);
  delete p;
}

extern "C" size_t fftgb_rplan_real_points(fftgb_rplan p) { return p ? p->real_points : 0; }

extern "C" size_t fftgb_rplan_spectrum_points(fftgb_rplan p) {
  return p ? p->spec_points : 0;
}

// column pass of length 2^log_l over the half-spectrum array
static cudaError_t cols(const float2 *in, float2 *out, int log_l, long long ncols,
                        long long inner, cudaStream_t s, int inverse, float scale) {
  ColsArgs a;
  a.in = in;
  a.out = out;
  a.ncols = ncols;
  a.inner = inner;
  a.tw = internal_axis_tw(log_l);
  a.tw4_lo = a.tw4_hi = NULL;
  a.tw4_bits = 0;
  a.scale = scale;
  a.swap_io = inverse;
  a.out_mode = 0;
  return launch_cols(log_l, a, s);
}

static int overlap(const void *a, size_t na, const void *b, size_t nb) {
  const char *x = (const char *)a, *y = (const char *)b;
  return x < y + nb && y < x + na;
}

extern "C" int fftgb_exec_r2c(fftgb_rplan p, const float *d_real, void *d_spectrum,
                              float scale, void *stream) {
  if (!p || !d_real || !d_spectrum) return FFTGB_EINVAL;
  if (overlap(d_real, p->real_points * 4, d_spectrum, p->spec_points * 8)) {
    internal_set_err("r2c input and output overlap");
    return FFTGB_EINVAL;
  }
  int device = 0;
  int rc = internal_ensure_device(&device);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned m = p->nx / 2;
  const long long w = m + 1;
  float2 *spec = (float2 *)d_spectrum;
  const bool last_x = p->ny == 1 && p->nz == 1;
  RealArgs a;
  a.in = (const float2 *)d_real;
  a.out = spec;
  a.nrows = (long long)p->ny * p->nz * p->batch;
  a.tw = internal_axis_tw(ilog2(m));
  a.wn = p->wn;
  a.scale = last_x ? scale : 1.0f;
  cudaError_t e;
  if (p->mx.n) {  // the packed rows' transform and the split in one pass
    e = mix_real_pass(p->mx, p->wn, (const float2 *)d_real, spec, a.nrows, 0, a.scale, s);
  } else {
    e = launch_r2c_rows(ilog2(m), a, s);
  }
  const long long planes = (long long)p->nz * p->batch;
  // the scale goes with the last pass
  const float sy = p->nz > 1 ? 1.0f : scale;
  if (e == cudaSuccess && p->ny > 1)
    e = p->my.n ? mix_pass(p->my, spec, spec, planes * w, w, 0, sy, s)
                : cols(spec, spec, ilog2(p->ny), planes * w, w, s, 0, sy);
  if (e == cudaSuccess && p->nz > 1) {
    const long long zl = (long long)p->batch * p->ny * w, zi = (long long)p->ny * w;
    e = p->mz.n ? mix_pass(p->mz, spec, spec, zl, zi, 0, scale, s)
                : cols(spec, spec, ilog2(p->nz), zl, zi, s, 0, scale);
  }
  if (e != cudaSuccess) {
    internal_set_err(cudaGetErrorString(e));
    return FFTGB_ECUDA;
  }
  return FFTGB_OK;
}

extern "C" int fftgb_exec_c2r(fftgb_rplan p, const void *d_spectrum, float *d_real,
                              float scale, void *stream) {
  if (!p || !d_spectrum || !d_real) return FFTGB_EINVAL;
  if (overlap(d_real, p->real_points * 4, d_spectrum, p->spec_points * 8)) {
    internal_set_err("c2r input and output overlap");
    return FFTGB_EINVAL;
  }
  int device = 0;
  int rc = internal_ensure_device(&device);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned m = p->nx / 2;
  const long long w = m + 1;
  const float2 *src = (const float2 *)d_spectrum;
  cudaError_t e = cudaSuccess;
  if (p->nz > 1) {
    const long long zl = (long long)p->batch * p->ny * w, zi = (long long)p->ny * w;
    e = p->mz.n ? mix_pass(p->mz, src, p->scratch, zl, zi, 1, 1.0f, s)
                : cols(src, p->scratch, ilog2(p->nz), zl, zi, s, 1, 1.0f);
    src = p->scratch;
  }
  if (e == cudaSuccess && p->ny > 1) {
    const long long yl = (long long)p->nz * p->batch * w;
    e = p->my.n ? mix_pass(p->my, src, p->scratch, yl, w, 1, 1.0f, s)
                : cols(src, p->scratch, ilog2(p->ny), yl, w, s, 1, 1.0f);
    src = p->scratch;
  }
  if (e == cudaSuccess) {
    RealArgs a;
    a.in = src;
    a.out = (float2 *)d_real;
    a.nrows = (long long)p->ny * p->nz * p->batch;
    a.tw = internal_axis_tw(ilog2(m));
    a.wn = p->wn;
    a.scale = scale;
    if (p->mx.n) {  // the combination and the inverse transform in one pass
      e = mix_real_pass(p->mx, p->wn, src, (float2 *)d_real, a.nrows, 1, scale, s);
    } else {
      e = launch_c2r_rows(ilog2(m), a, s);
    }
  }
  if (e != cudaSuccess) {
    internal_set_err(cudaGetErrorString(e));
    return FFTGB_ECUDA;
  }
  return FFTGB_OK;
}
