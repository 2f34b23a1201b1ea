// spectral.cu - element-wise kernels around the transforms (spectral.cuh).
// Both are single HBM streams (every point read once, written at most once)
// with grid-stride loops over a grid of a few CTAs per SM.
#include "fft_core.cuh"
#include "filter.cuh"
#include "spectral.cuh"

namespace fftgb {

namespace {
constexpr int SP_THREADS = 256;

// SMs of the current device, queried once per device (a few CTAs per SM)
int sp_sms() {
  constexpr int kMaxDev = 64;
  static int cached[kMaxDev] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return 152;
  if (!cached[dev]) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        sms < 1)
      return 152;
    cached[dev] = sms;
  }
  return cached[dev];
}

int sp_grid(long long n) {
  const int sms = sp_sms();
  const long long need = (n + SP_THREADS - 1) / SP_THREADS;
  const long long cap = (long long)sms * 8;
  return (int)(need < cap ? (need > 0 ? need : 1) : cap);
}
}  // namespace

// POW2: sides powers of two (log2 lx, ly, lz: masks and shifts); otherwise
// any sides, the batch below 2^32 points (32-bit divisions).
template <bool POW2>
__global__ void __launch_bounds__(SP_THREADS) k_filter(float2 *d, long long n, int nx, int ny,
                                                       int nz, int lx, int ly, int kind) {
  for (long long i = blockIdx.x * (long long)SP_THREADS + threadIdx.x; i < n;
       i += (long long)gridDim.x * SP_THREADS) {
    int kx, ky, kz;
    if (POW2) {
      kx = (int)(i & (nx - 1));
      ky = (int)((i >> lx) & (ny - 1));
      kz = (int)((i >> (lx + ly)) & (nz - 1));
    } else {
      unsigned u = (unsigned)i % ((unsigned)nx * (unsigned)ny * (unsigned)nz);
      kx = (int)(u % (unsigned)nx);
      u /= (unsigned)nx;
      ky = (int)(u % (unsigned)ny);
      kz = (int)(u / (unsigned)ny);
    }
    d[i] = cscale(d[i], filter_g(kind, kx, ky, kz, nx, ny, nz));
  }
}

__global__ void __launch_bounds__(SP_THREADS) k_sq_residual(const float2 *__restrict__ a,
                                                            const float2 *__restrict__ b,
                                                            float2 *__restrict__ r, long long n,
                                                            double *sum) {
  __shared__ double part[SP_THREADS / 32];
  float acc = 0.0f;
  for (long long i = blockIdx.x * (long long)SP_THREADS + threadIdx.x; i < n;
       i += (long long)gridDim.x * SP_THREADS) {
    const float2 d = csub(a[i], b[i]);
    if (r) r[i] = d;
    acc = fmaf(d.x, d.x, fmaf(d.y, d.y, acc));
  }
  double w = acc;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = w;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
#pragma unroll
    for (int k = 0; k < SP_THREADS / 32; k++) t += part[k];
    atomicAdd(sum, t);
  }
}

static bool pow2i(int v) { return v > 0 && !(v & (v - 1)); }
static int log2i(int v) {
  int r = 0;
  while ((1 << r) < v) r++;
  return r;
}

cudaError_t launch_filter(float2 *d, long long points, int nx, int ny, int nz, int kind,
                          cudaStream_t s) {
  if (points <= 0) return cudaSuccess;
  if (nx < 1 || ny < 1 || nz < 1) return cudaErrorInvalidValue;
  if (pow2i(nx) && pow2i(ny) && pow2i(nz)) {
    k_filter<true><<<sp_grid(points), SP_THREADS, 0, s>>>(d, points, nx, ny, nz, log2i(nx),
                                                          log2i(ny), kind);
  } else {
    if (points >= (1LL << 32)) return cudaErrorInvalidValue;
    k_filter<false><<<sp_grid(points), SP_THREADS, 0, s>>>(d, points, nx, ny, nz, 0, 0, kind);
  }
  return cudaGetLastError();
}

cudaError_t launch_sq_residual(const float2 *a, const float2 *b, float2 *r, long long n,
                               double *sum, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_sq_residual<<<sp_grid(n), SP_THREADS, 0, s>>>(a, b, r, n, sum);
  return cudaGetLastError();
}

}  // namespace fftgb
