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
#include "tc_core.cuh"

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

// ---------------------------------------------------------------------------
// Bulk-copy exchange (k_1d_push).  Same algorithm and outputs as k_1d_cluster,
// but the four-step transpose is pushed, not pulled: after step 1 CTA c holds
// Y[k2][n1 local] for all k2, and the rows owned by CTA d (k2 in
// [d*ROWS, (d+1)*ROWS)) are one contiguous ROWS*COLS block of it.  One thread
// per destination sends that block with cp.async.bulk into d's receive area
// (block-major: [source c][row][column]); the copy completes on d's own
// mbarrier, which expects C blocks.  So no CTA reads remote shared memory and
// no cluster barrier sits between the two steps:
//   * a split cluster barrier (arrive at entry, wait before the first send)
//     publishes every CTA's initialised mbarrier; step 1 runs inside it;
//   * a second split barrier (arrive once this CTA has received everything,
//     wait before exit) keeps every CTA resident until all copies, which read
//     the sender's shared memory, have landed.
// Sends are staggered (CTA c's j-th copy goes to CTA (c + j) % C) so that no
// CTA receives from every sender at once.
template <int L1, int L2, int C>
struct C1pCfg {
  using K = C1dCfg<L1, L2, C>;
  static constexpr int YPTS = L2 * K::COLS;           // send area, points
  static constexpr int RPTS = K::ROWS * K::RS;        // receive area, points
  static constexpr int BLOCK = K::ROWS * K::COLS;     // points per copy
  static constexpr int BLOCK_BYTES = BLOCK * (int)sizeof(float2);
  static constexpr int MBAR_OFF = (YPTS + RPTS) * (int)sizeof(float2);
  static constexpr int SMEM = MBAR_OFF + 16;
  static_assert(BLOCK_BYTES % 16 == 0 && (YPTS * (int)sizeof(float2)) % 16 == 0,
                "bulk copies move 16-byte multiples between 16-byte aligned addresses");
  static_assert(MBAR_OFF % 8 == 0, "mbarrier alignment");
  static_assert(C * BLOCK_BYTES < (1 << 20), "mbarrier transaction count range");
  static_assert(C <= K::THREADS, "one sending thread per destination");
};

constexpr uint32_t C1P_WAIT_LIMIT = 1u << 22;
static __device__ int g_c1d_status;
__global__ void k_cluster1d_expire(uint32_t polls) { tc::expire_wait(&g_c1d_status, polls); }

__device__ __forceinline__ uint32_t cluster_map(uint32_t a, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ void cluster_arrive_relaxed() {
  asm volatile("barrier.cluster.arrive.relaxed.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() {
  asm volatile("barrier.cluster.wait.aligned;\n" ::: "memory");
}

template <int L1, int L2, int C, bool INV>
__global__ void __cluster_dims__(C, 1, 1)
    __launch_bounds__(C1dCfg<L1, L2, C>::THREADS,
                      C1dCfg<L1, L2, C>::THREADS <= 256 ? 3 : 1)
    k_1d_push(const C1dArgs a) {
  using K = C1dCfg<L1, L2, C>;
  using P = C1pCfg<L1, L2, C>;
  using CA = typename K::CA;
  using CB = typename K::CB;
  constexpr int E = K::E, N = K::N, COLS = K::COLS, ROWS = K::ROWS, RS = K::RS;
  extern __shared__ __align__(128) unsigned char c1p_smem[];
  float2 *Y = reinterpret_cast<float2 *>(c1p_smem);
  float2 *R = Y + P::YPTS;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(c1p_smem + P::MBAR_OFF);
  const int c = (int)cg::this_cluster().block_rank();
  const long long tr = blockIdx.x / C;
  const int tid = threadIdx.x;

  if (tid == 0) {
    tc::mbar_init(mbar, 1);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(
                     tc::smem_u32(mbar)),
                 "r"((uint32_t)(C * P::BLOCK_BYTES))
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  cluster_arrive_relaxed();

  // ---- step 1: column FFTs over n2 (stride L1), twiddle W_N^(n1*k2)
  {
    const float2 *src = a.in + tr * N;
    const int cl = tid % COLS;
    const int t = tid / COLS;
    const int n1 = c * COLS + cl;
    float2 v[E];
#pragma unroll
    for (int q = 0; q < E; q++) {
      const float2 x = src[n1 + (long long)L1 * in_index<CA>(t, q)];
      v[q] = INV ? cswap(x) : x;
    }
    stockham<CA>(v, t, [Y, cl](int i) -> float2 & { return Y[i * COLS + cl]; }, a.tw_a);
    if (CA::NSTG > 1) __syncthreads();
#pragma unroll
    for (int q = 0; q < E; q++) {
      const int k2 = out_index<CA>(t, q);
      Y[k2 * COLS + cl] =
          cmul(v[q], twiddle2(a.tw4_lo, a.tw4_hi, a.tw4_bits, (long long)n1 * k2));
    }
  }
  tc::fence_proxy_async();  // the copies read Y through the async proxy
  __syncthreads();
  cluster_wait();  // every CTA's mbarrier is initialised
  if (tid < C) {
    const int d = (c + tid) % C;
    const uint32_t src = tc::smem_u32(Y + d * P::BLOCK);
    const uint32_t dst = cluster_map(tc::smem_u32(R + c * P::BLOCK), (uint32_t)d);
    const uint32_t mb = cluster_map(tc::smem_u32(mbar), (uint32_t)d);
    asm volatile(
        "cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes "
        "[%0], [%1], %2, [%3];\n" ::"r"(dst),
        "r"(src), "r"((uint32_t)P::BLOCK_BYTES), "r"(mb)
        : "memory");
  }
  const bool got = tc::mbar_wait_bounded(mbar, 0, C1P_WAIT_LIMIT);
  cluster_arrive_relaxed();  // this CTA's receive area is complete
  if (!__syncthreads_and(got)) {
    if (tid == 0) atomicExch(&g_c1d_status, 1);
    cluster_wait();
    return;
  }

  // ---- step 2: rows k2 from the receive area, FFT over n1, store
  const int rl = tid / CB::T;
  const int t = tid % CB::T;
  const int k2 = c * ROWS + rl;
  float2 v[E];
#pragma unroll
  for (int q = 0; q < E; q++) {
    const int n1 = in_index<CB>(t, q);
    v[q] = R[(n1 / COLS) * P::BLOCK + rl * COLS + (n1 % COLS)];
  }
  __syncthreads();  // the receive area becomes the rows' scratch
  float2 *row = R + rl * RS;
  stockham<CB>(v, t, [row](int i) -> float2 & { return row[swz(i)]; }, a.tw_b);
  if (CB::NSTG > 1) __syncthreads();
#pragma unroll
  for (int q = 0; q < E; q++) row[swz(out_index<CB>(t, q))] = v[q];
  __syncthreads();
  float2 *dst = a.out + tr * N;
  if (a.bitrev) {
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
#pragma unroll
    for (int q = 0; q < E; q++) {
      const int p = tid + q * K::THREADS;  // p = k1*ROWS + r
      const int k1 = p / ROWS;
      const int r = p - k1 * ROWS;
      float2 x = R[r * RS + swz(k1)];
      if (a.scale != 1.0f) x = cscale(x, a.scale);
      dst[(long long)k1 * L2 + c * ROWS + r] = INV ? cswap(x) : x;
    }
  }
  cluster_wait();  // all copies out of this CTA's send area have landed
}

namespace {
struct C1dEntry {
  int n;
  int l1, l2, c;
  void (*fn[2])(const C1dArgs);  // [inverse]
  int threads, smem;
  void (*fnp[2])(const C1dArgs);  // bulk-copy exchange form, or null
  int smemp;
  int push_default;  // the bulk-copy form is the measured default
};
#define C1D(L1, L2, C)                                                    \
  {L1 * L2, L1, L2, C,                                                    \
   {k_1d_cluster<L1, L2, C, false>, k_1d_cluster<L1, L2, C, true>},        \
   C1dCfg<L1, L2, C>::THREADS, C1dCfg<L1, L2, C>::SMEM, {nullptr, nullptr}, 0, 0}
#define C1DP(L1, L2, C, DEF)                                              \
  {L1 * L2, L1, L2, C,                                                    \
   {k_1d_cluster<L1, L2, C, false>, k_1d_cluster<L1, L2, C, true>},        \
   C1dCfg<L1, L2, C>::THREADS, C1dCfg<L1, L2, C>::SMEM,                   \
   {k_1d_push<L1, L2, C, false>, k_1d_push<L1, L2, C, true>},              \
   C1pCfg<L1, L2, C>::SMEM, DEF}
// The first entry of each n is its default; the others are tuning choices.
// Bulk-copy forms, measured on GB300 against the remote-load form: 65536
// points on 16-CTA clusters x 8: 0.0103 against 0.0123 ms, x 32 and above
// equal within 3 %, so it is the default there; 32768 points on 8-CTA
// clusters x 64: 0.0185 against 0.0165 ms, x 2048: 0.373 against 0.344 ms
// (three CTAs per SM instead of four), so it is not.
const C1dEntry kC1d[] = {
    C1D(256, 256, 4),
    C1D(256, 256, 8),
    C1DP(256, 256, 16, 1),
    C1D(256, 128, 2),
    C1DP(256, 128, 8, 0),
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
      if (e.fnp[d]) {
        r = cudaFuncSetAttribute((const void *)e.fnp[d],
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, e.smemp);
        if (r == cudaSuccess && e.c > 8)
          r = cudaFuncSetAttribute((const void *)e.fnp[d],
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
      if (a.push && e.fnp[0])
        e.fnp[a.swap_io ? 1 : 0]<<<(unsigned)grid, e.threads, e.smemp, s>>>(a);
      else
        e.fn[a.swap_io ? 1 : 0]<<<(unsigned)grid, e.threads, e.smem, s>>>(a);
      return cudaGetLastError();
    }
  }
  return cudaErrorInvalidValue;
}

int cluster1d_exchange_forms(int n, int c) {
  for (const C1dEntry &e : kC1d)
    if (e.n == n && (c == 0 || e.c == c))
      return 1 | (e.fnp[0] ? 2 : 0) | (e.push_default ? 4 : 0);
  return 0;
}

cudaError_t cluster1d_expire_wait(unsigned polls) {
  k_cluster1d_expire<<<1, 32>>>(polls);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? cudaDeviceSynchronize() : e;
}

int cluster1d_status_and_clear() {
  int st = 0;
  const int zero = 0;
  if (cudaMemcpyFromSymbol(&st, g_c1d_status, sizeof(int)) != cudaSuccess) return -1;
  if (st && cudaMemcpyToSymbol(g_c1d_status, &zero, sizeof(int)) != cudaSuccess) return -1;
  return st;
}

}  // namespace fftgb
