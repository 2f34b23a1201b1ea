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
#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>

#include <vector>

#include "fftfpga_ext.h"
#include "../kernels/fft_pass.cuh"
#include "../kernels/fft_real.cuh"

namespace fftgb {
int internal_ensure_device(int *device);
const float2 *internal_axis_tw(int log_l);
void internal_set_err(const char *msg);
}  // namespace fftgb

using namespace fftgb;

struct fftgb_rplan_s {
  int rank;
  unsigned nx, ny, nz, batch;
  size_t real_points, spec_points;
  float2 *wn;       // W_nx^k, k = 0..nx/2
  float2 *scratch;  // C2R with y or z passes: half-spectrum work buffer
};

static int ilog2(unsigned v) {
  int r = 0;
  while ((1u << r) < v) r++;
  return r;
}

static bool pow2(unsigned v) { return v && !(v & (v - 1)); }

extern "C" int fftgb_plan_r2c(fftgb_rplan *plan, int rank, unsigned nx, unsigned ny,
                              unsigned nz, unsigned batch) {
  if (!plan) return FFTGB_EINVAL;
  *plan = NULL;
  if (rank < 1 || rank > 3 || batch == 0 || (rank < 2 && ny != 1) ||
      (rank < 3 && nz != 1) || !pow2(nx) || !pow2(ny) || !pow2(nz)) {
    internal_set_err("r2c plan: rank 1-3, power-of-two sizes, unused sizes 1, batch > 0");
    return FFTGB_EINVAL;
  }
  if (nx < 4 || nx > 8192 || ny > 4096 || nz > 4096) {
    internal_set_err("r2c plan: nx must be 4..8192 and ny, nz at most 4096");
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
  cudaError_t e = launch_r2c_rows(ilog2(m), a, s);
  const long long planes = (long long)p->nz * p->batch;
  // the scale goes with the last pass
  if (e == cudaSuccess && p->ny > 1)
    e = cols(spec, spec, ilog2(p->ny), planes * w, w, s, 0, p->nz > 1 ? 1.0f : scale);
  if (e == cudaSuccess && p->nz > 1)
    e = cols(spec, spec, ilog2(p->nz), (long long)p->batch * p->ny * w,
             (long long)p->ny * w, s, 0, scale);
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
    e = cols(src, p->scratch, ilog2(p->nz), (long long)p->batch * p->ny * w,
             (long long)p->ny * w, s, 1, 1.0f);
    src = p->scratch;
  }
  if (e == cudaSuccess && p->ny > 1) {
    e = cols(src, p->scratch, ilog2(p->ny), (long long)p->nz * p->batch * w, w, s, 1, 1.0f);
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
    e = launch_c2r_rows(ilog2(m), a, s);
  }
  if (e != cudaSuccess) {
    internal_set_err(cudaGetErrorString(e));
    return FFTGB_ECUDA;
  }
  return FFTGB_OK;
}
