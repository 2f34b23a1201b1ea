// fft1d_cluster.cu - single-pass 1D FFT of N = L1*L2 points per transform on
// a thread-block cluster of C CTAs, the transpose of the four-step algorithm
// done through distributed shared memory instead of HBM.
//
// Replaces the reference's 1D path (kernels/fft1d/fft1d.cl:140-252), whose
// engine streams 8 points per cycle and stores the result bit-reversed.  A
// 65536-point transform (512 KiB) does not fit one SM's shared memory but
// fits four: each point then crosses HBM once on the way in and once on the
// way out (the two-pass four-step moves it twice each way).
//
// n = n1 + L1*n2, k = k2 + L2*k1:
//   step 1 (CTA c owns columns n1 in [c*L1/C, (c+1)*L1/C)): FFT over n2 of
//     every owned column, times W_N^(n1*k2), kept in the CTA's shared memory
//     as Y[k2][n1 local];
//   cluster barrier;
//   step 2 (CTA c owns rows k2 in [c*L2/C, (c+1)*L2/C)): gather Y[k2][n1] for
//     all n1 from the owning CTAs' shared memory (distributed shared memory
//     loads), cluster barrier, FFT over n1, store X[k2 + L2*k1] (natural) or
//     at bitrev(k2 + L2*k1) (the fftfpgaf_c2c_1d order).
#include <cooperative_groups.h>

#include "fft_core.cuh"
#include "fft1d_cluster.cuh"

namespace cg = cooperative_groups;

namespace fftgb {

template <int L1, int L2, int C>
struct C1dCfg {
  static constexpr int E = 16;
  static constexpr int N = L1 * L2;
  static constexpr int COLS = L1 / C;  // step-1 columns per CTA
  static constexpr int ROWS = L2 / C;  // step-2 rows per CTA
  using CA = Stock<L2, E>;             // over n2
  using CB = Stock<L1, E>;             // over n1
  static constexpr int THREADS = COLS * CA::T;
  static_assert(THREADS == ROWS * CB::T, "step thread counts differ");
  static_assert(THREADS <= 1024, "too many threads");
  static constexpr int RS = L1 + 1;  // padded row stride of step 2
  static constexpr int S1 = L2 * COLS;
  static constexpr int S2 = ROWS * RS;
  static constexpr int SMEM = (S1 > S2 ? S1 : S2) * (int)sizeof(float2);
};

// CTAs of 512 threads or fewer are held to 64 registers so that two or more
// clusters share an SM and overlap their load, exchange and store phases.
template <int L1, int L2, int C, bool INV>
__global__ void __cluster_dims__(C, 1, 1)
    __launch_bounds__(C1dCfg<L1, L2, C>::THREADS,
                      C1dCfg<L1, L2, C>::THREADS <= 512 ? 1024 / C1dCfg<L1, L2, C>::THREADS : 1)
    k_1d_cluster(const C1dArgs a) {
  using K = C1dCfg<L1, L2, C>;
  using CA = typename K::CA;
  using CB = typename K::CB;
  constexpr int E = K::E, N = K::N, COLS = K::COLS, ROWS = K::ROWS, RS = K::RS;
  extern __shared__ float2 smem[];
  cg::cluster_group cluster = cg::this_cluster();
  const int c = (int)cluster.block_rank();
  const long long tr = blockIdx.x / C;  // transform index in the batch
  const int tid = threadIdx.x;
  const float2 *src = a.in + tr * N;

  // ---- step 1: column FFTs over n2 (stride L1), twiddle W_N^(n1*k2)
  {
    const int cl = tid % COLS;
    const int t = tid / COLS;
    const int n1 = c * COLS + cl;
    float2 v[E];
#pragma unroll
    for (int q = 0; q < E; q++) {
      const float2 x = src[n1 + (long long)L1 * in_index<CA>(t, q)];
      v[q] = INV ? cswap(x) : x;
    }
    stockham<CA>(v, t, [cl](int i) -> float2 & {
      extern __shared__ float2 s_[];
      return s_[i * COLS + cl];
    }, a.tw_a);
    if (CA::NSTG > 1) __syncthreads();
#pragma unroll
    for (int q = 0; q < E; q++) {
      const int k2 = out_index<CA>(t, q);
      smem[k2 * COLS + cl] =
          cmul(v[q], twiddle2(a.tw4_lo, a.tw4_hi, a.tw4_bits, (long long)n1 * k2));
    }
  }
  cluster.sync();

  // ---- step 2: gather rows k2 from the owners, FFT over n1, store
  const int rl = tid / CB::T;
  const int t = tid % CB::T;
  const int k2 = c * ROWS + rl;
  float2 v[E];
#pragma unroll
  for (int q = 0; q < E; q++) {
    const int n1 = in_index<CB>(t, q);
    const float2 *owner = cluster.map_shared_rank(smem, n1 / COLS);
    v[q] = owner[k2 * COLS + (n1 % COLS)];
  }
  cluster.sync();  // every remote read done before shared memory is reused
  float2 *row = smem + rl * RS;
  stockham<CB>(v, t, [row](int i) -> float2 & { return row[swz(i)]; }, a.tw_b);
  if (CB::NSTG > 1) __syncthreads();
#pragma unroll
  for (int q = 0; q < E; q++) row[swz(out_index<CB>(t, q))] = v[q];
  __syncthreads();
  float2 *dst = a.out + tr * N;
  if (a.bitrev) {
    // bitrev(k2 + L2*k1) = bitrev_a(k1) + L1*bitrev_b(k2): row bitrev_b(k2),
    // bit-reversed order within the row
    constexpr int LA = ilog2c(L1), LB = ilog2c(L2);
    float2 *drow = dst + (long long)bitrev_n((unsigned)k2, LB) * L1;
#pragma unroll
    for (int q = 0; q < E; q++) {
      const int p = t + q * CB::T;
      float2 x = row[swz((int)bitrev_n((unsigned)p, LA))];
      if (a.scale != 1.0f) x = cscale(x, a.scale);
      drow[p] = INV ? cswap(x) : x;
    }
  } else {
    // natural: X[k2 + L2*k1]; ROWS consecutive k2 per k1 are contiguous
#pragma unroll
    for (int q = 0; q < E; q++) {
      const int p = tid + q * K::THREADS;  // p = k1*ROWS + r
      const int k1 = p / ROWS;
      const int r = p - k1 * ROWS;
      float2 x = smem[r * RS + swz(k1)];
      if (a.scale != 1.0f) x = cscale(x, a.scale);
      dst[(long long)k1 * L2 + c * ROWS + r] = INV ? cswap(x) : x;
    }
  }
}

namespace {
struct C1dEntry {
  int n;
  int l1, l2, c;
  void (*fn[2])(const C1dArgs);  // [inverse]
  int threads, smem;
};
#define C1D(L1, L2, C)                                                    \
  {L1 * L2, L1, L2, C,                                                    \
   {k_1d_cluster<L1, L2, C, false>, k_1d_cluster<L1, L2, C, true>},        \
   C1dCfg<L1, L2, C>::THREADS, C1dCfg<L1, L2, C>::SMEM}
// The first entry of each n is its default; the others are tuning choices.
const C1dEntry kC1d[] = {
    C1D(256, 256, 4),
    C1D(256, 256, 8),
    C1D(256, 256, 16),
    C1D(256, 128, 2),
    C1D(256, 128, 8),
    C1D(512, 256, 8),
    C1D(512, 256, 16),
};
bool g_c1d_ready = false;
}  // namespace

cudaError_t cluster1d_init() {
  if (g_c1d_ready) return cudaSuccess;
  for (const C1dEntry &e : kC1d) {
    for (int d = 0; d < 2; d++) {
      cudaError_t r = cudaFuncSetAttribute(
          (const void *)e.fn[d], cudaFuncAttributeMaxDynamicSharedMemorySize,
          e.smem);
      if (r != cudaSuccess) return r;
      if (e.c > 8) {  // 16-CTA clusters are a non-portable size
        r = cudaFuncSetAttribute((const void *)e.fn[d],
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (r != cudaSuccess) return r;
      }
    }
  }
  g_c1d_ready = true;
  return cudaSuccess;
}

bool cluster1d_available(int n, int c, int *l1, int *l2) {
  for (const C1dEntry &e : kC1d) {
    if (e.n == n && (c == 0 || e.c == c)) {
      if (l1) *l1 = e.l1;
      if (l2) *l2 = e.l2;
      return true;
    }
  }
  return false;
}

int cluster1d_sizes(int n, int *sizes, int max_sizes) {
  int k = 0;
  for (const C1dEntry &e : kC1d)
    if (e.n == n && k < max_sizes) sizes[k++] = e.c;
  return k;
}

cudaError_t launch_cluster1d(int n, int c, const C1dArgs &a, cudaStream_t s) {
  if (!g_c1d_ready) return cudaErrorInvalidValue;
  for (const C1dEntry &e : kC1d) {
    if (e.n == n && (c == 0 || e.c == c)) {
      const long long grid = a.count * e.c;
      if (grid <= 0 || grid > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
      e.fn[a.swap_io ? 1 : 0]<<<(unsigned)grid, e.threads, e.smem, s>>>(a);
      return cudaGetLastError();
    }
  }
  return cudaErrorInvalidValue;
}

}  // namespace fftgb
