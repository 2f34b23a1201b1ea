// fft_real.cu - the contiguous-axis pass of real-data transforms (R2C and
// C2R), for real rows of N = 2M points.  The reference has no real-data
// transforms (its README lists them as missing); the layout follows the
// common half-spectrum convention: a row of N reals <-> M + 1 complex values
// X[0..M], the inverse unnormalised (C2R(R2C(x)) = N x).
//
// R2C: the row is read as M complex points z[n] = x[2n] + i x[2n+1] (no
// copy), Z = DFT_M(z) runs in registers (Stockham, as k_rows), and
//   E[k] = (Z[k] + conj Z[M-k]) / 2,  O[k] = (Z[k] - conj Z[M-k]) / (2i),
//   X[k] = E[k] + W_N^k O[k],  k = 0..M  (Z[M] = Z[0]),
// is formed from the natural-order result in shared memory.
// C2R: Z'[k] = (X[k] + conj X[M-k]) + i W_N^-k (X[k] - conj X[M-k]) for
// k < M, then the unnormalised inverse DFT_M gives z'[n] = N (x[2n] +
// i x[2n+1]), stored as the real row.
#include "fft_core.cuh"
#include "fft_real.cuh"

namespace fftgb {

template <int M>
struct RealCfg {
  using C = Cfg<M>;
  static constexpr int THREADS = (M >= 256) ? 512 : 256;
  static constexpr int F = THREADS / C::T;  // rows per CTA
  static constexpr int SMEM = F * M * (int)sizeof(float2);
};

template <int M>
__global__ void __launch_bounds__(RealCfg<M>::THREADS, RealCfg<M>::THREADS == 512 ? 2 : 1)
    k_r2c_rows(const RealArgs a) {
  using C = Cfg<M>;
  constexpr int T = C::T, E = C::E, F = RealCfg<M>::F;
  extern __shared__ float2 smem[];
  const int tid = threadIdx.x;
  const int fl = tid / T;
  const int t = tid - fl * T;
  const long long row = (long long)blockIdx.x * F + fl;
  const bool ok = row < a.nrows;
  const float2 *src = a.in + row * M;
  float2 v[E];
#pragma unroll
  for (int q = 0; q < E; q++)
    v[q] = ok ? src[in_index<C>(t, q)] : make_float2(0.f, 0.f);
  float2 *mysm = smem + fl * M;
  auto sm = [mysm](int i) -> float2 & { return mysm[swz(i)]; };
  stockham<C>(v, t, sm, a.tw);
  __syncthreads();  // last exchange reads done before the result overwrites
#pragma unroll
  for (int q = 0; q < E; q++) sm(out_index<C>(t, q)) = v[q];
  __syncthreads();
  if (!ok) return;
  float2 *dst = a.out + row * (M + 1);
#pragma unroll
  for (int j = 0; j <= E; j++) {
    const int k = t + j * T;  // 0..M (k == M only for t == 0, j == E)
    if (j == E && t != 0) break;
    const float2 zk = sm(k & (M - 1));
    const float2 zm = sm((M - k) & (M - 1));
    const float2 e = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
    const float2 o = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
    float2 x = cadd(e, cmul(__ldg(&a.wn[k]), o));
    if (a.scale != 1.0f) x = cscale(x, a.scale);
    dst[k] = x;
  }
}

template <int M>
__global__ void __launch_bounds__(RealCfg<M>::THREADS, RealCfg<M>::THREADS == 512 ? 2 : 1)
    k_c2r_rows(const RealArgs a) {
  using C = Cfg<M>;
  constexpr int T = C::T, E = C::E, F = RealCfg<M>::F;
  extern __shared__ float2 smem[];
  const int tid = threadIdx.x;
  const int fl = tid / T;
  const int t = tid - fl * T;
  const long long row = (long long)blockIdx.x * F + fl;
  const bool ok = row < a.nrows;
  const float2 *src = a.in + row * (M + 1);
  float2 v[E];
#pragma unroll
  for (int q = 0; q < E; q++) {
    const int k = in_index<C>(t, q);
    float2 z = make_float2(0.f, 0.f);
    if (ok) {
      const float2 xk = src[k], xm = src[M - k];
      const float2 s = make_float2(xk.x + xm.x, xk.y - xm.y);
      const float2 d = make_float2(xk.x - xm.x, xk.y + xm.y);
      const float2 w = __ldg(&a.wn[k]);
      const float2 dw = cmul(d, make_float2(w.x, -w.y));  // W_N^-k
      z = make_float2(s.x - dw.y, s.y + dw.x);            // s + i dw
    }
    v[q] = cswap(z);  // inverse through the real/imaginary swap
  }
  float2 *mysm = smem + fl * M;
  stockham<C>(v, t, [mysm](int i) -> float2 & { return mysm[swz(i)]; }, a.tw);
  if (!ok) return;
  float2 *dst = a.out + row * M;
#pragma unroll
  for (int q = 0; q < E; q++) {
    float2 z = cswap(v[q]);
    if (a.scale != 1.0f) z = cscale(z, a.scale);
    dst[out_index<C>(t, q)] = z;
  }
}

namespace {
typedef void (*RealFn)(const RealArgs);
constexpr int MAXLOG = 12;
RealFn g_r2c[MAXLOG + 1], g_c2r[MAXLOG + 1];
int g_smem[MAXLOG + 1], g_thr[MAXLOG + 1], g_f[MAXLOG + 1];
bool g_real_ready = false;

template <int LOG>
struct RTab {
  static constexpr int M = 1 << LOG;
  static void fill() {
    g_r2c[LOG] = k_r2c_rows<M>;
    g_c2r[LOG] = k_c2r_rows<M>;
    g_smem[LOG] = RealCfg<M>::SMEM;
    g_thr[LOG] = RealCfg<M>::THREADS;
    g_f[LOG] = RealCfg<M>::F;
    RTab<LOG - 1>::fill();
  }
};
template <>
struct RTab<0> {
  static void fill() {}
};

cudaError_t launch(RealFn *tab, int log_m, const RealArgs &a, cudaStream_t s) {
  if (!g_real_ready || log_m < 1 || log_m > MAXLOG) return cudaErrorInvalidValue;
  const long long grid = (a.nrows + g_f[log_m] - 1) / g_f[log_m];
  if (grid <= 0 || grid > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  tab[log_m]<<<(unsigned)grid, g_thr[log_m], g_smem[log_m], s>>>(a);
  return cudaGetLastError();
}
}  // namespace

cudaError_t real_kernels_init() {
  if (g_real_ready) return cudaSuccess;
  RTab<MAXLOG>::fill();
  for (int l = 1; l <= MAXLOG; l++) {
    for (RealFn f : {g_r2c[l], g_c2r[l]}) {
      const cudaError_t e = cudaFuncSetAttribute(
          (const void *)f, cudaFuncAttributeMaxDynamicSharedMemorySize, g_smem[l]);
      if (e != cudaSuccess) return e;
    }
  }
  g_real_ready = true;
  return cudaSuccess;
}

cudaError_t launch_r2c_rows(int log_m, const RealArgs &a, cudaStream_t s) {
  return launch(g_r2c, log_m, a, s);
}

cudaError_t launch_c2r_rows(int log_m, const RealArgs &a, cudaStream_t s) {
  return launch(g_c2r, log_m, a, s);
}

}  // namespace fftgb
