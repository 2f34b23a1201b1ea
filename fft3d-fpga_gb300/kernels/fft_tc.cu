// fft_tc.cu - tensor-core split-precision form of the axis passes.
//
// The radix-16 stages of a Stockham FFT with 16 points per thread give each
// thread exactly one butterfly, so the 128 threads of a warpgroup hold 128
// butterflies: one dense product D[128 x 32] = A[128 x 32] * B[32 x 32]^T in
// real form (A row = a butterfly's twiddled inputs, re[0..15] im[0..15];
// B = the 16-point DFT matrix as a 32 x 32 real matrix).  One elected thread
// issues tcgen05.mma (kind::f16) with both operands in shared memory and the
// FP32 accumulators in TMEM; every thread then reads its own TMEM lane,
// which is its butterfly's 16 complex outputs.
//
// Precision: each butterfly is scaled by a power of two to bring its largest
// component to [1, 2), then split into half-precision terms:
//   FP16 mode: x = hi + lo, B = hi + lo, 3 products (hi*hi + lo*hi + hi*lo)
//   BF16 mode: x = hi + mid + lo, B likewise, 6 products (all pairs whose
//              term orders sum to <= 2)
// accumulated in FP32.  Twiddles stay in FP32 from the FP64-generated
// tables; the radix-2/4/8 stages stay on the FP32 cores.
#include <stdio.h>

#include "fft_core.cuh"
#include "fft_tc.cuh"
#include "tc_core.cuh"

namespace fftgb {

namespace {
constexpr int A_PLANE = 128 * 32 * 2;  // bytes of one A term plane
constexpr int B_PLANE = 32 * 32 * 2;   // bytes of one B term plane
constexpr uint32_t WAIT_LIMIT = 1u << 24;

__host__ __device__ constexpr int align1k(int x) { return (x + 1023) & ~1023; }
}  // namespace

// DFT16 in real form, FP32 values of FP64 cos/sin (set by tc_kernels_init)
static __device__ float g_tc_bmat[32 * 32];
// set to 1 when a tensor-core wait gave up
static __device__ int g_tc_status;
__global__ void k_tc_expire(uint32_t polls) { tc::expire_wait(&g_tc_status, polls); }

__device__ __forceinline__ void wg_bar(int id) {
  asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(128) : "memory");
}

template <int MODE>
struct TcTerms {
  static constexpr int NP = (MODE == 1) ? 2 : 3;
};

template <int MODE>
__device__ __forceinline__ void store_terms(uint8_t *base, int plane_bytes, int off,
                                            float x) {
  if constexpr (MODE == 1) {
    __half h, l;
    tc::split_f16(x, h, l);
    *(__half *)(base + off) = h;
    *(__half *)(base + plane_bytes + off) = l;
  } else {
    __nv_bfloat16 h, m, l;
    tc::split_bf16(x, h, m, l);
    *(__nv_bfloat16 *)(base + off) = h;
    *(__nv_bfloat16 *)(base + plane_bytes + off) = m;
    *(__nv_bfloat16 *)(base + 2 * plane_bytes + off) = l;
  }
}

// Radix-16 butterfly of one thread, evaluated with its warpgroup on the
// tensor cores.  All 128 threads of the warpgroup must call it together.
template <int MODE>
struct TcRadix16 {
  uint8_t *sa;        // this warpgroup's A term planes
  const uint8_t *sb;  // B term planes (shared by the CTA)
  uint64_t *mbar;     // this warpgroup's MMA-completion barrier
  uint32_t tcol;      // TMEM address of this warpgroup's 32 columns
  uint32_t phase;
  int r;              // row of this thread = its TMEM lane
  int bar_id;         // named barrier of the warpgroup

  __device__ __forceinline__ void operator()(float2 *v) {
    constexpr int NP = TcTerms<MODE>::NP;
    float m = 0.f;
#pragma unroll
    for (int k = 0; k < 16; k++) m = fmaxf(m, fmaxf(fabsf(v[k].x), fabsf(v[k].y)));
    int e = (int)((__float_as_uint(m) >> 23) & 0xff) - 127;
    e = max(-100, min(100, e));
    const float s = __uint_as_float((uint32_t)(127 - e) << 23);
    const float us = __uint_as_float((uint32_t)(127 + e) << 23);
#pragma unroll
    for (int k = 0; k < 16; k++) {
      store_terms<MODE>(sa, A_PLANE, tc::core_off(r, k, 32), v[k].x * s);
      store_terms<MODE>(sa, A_PLANE, tc::core_off(r, 16 + k, 32), v[k].y * s);
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    wg_bar(bar_id);
    tc::fence_after_sync();
    if (r == 0) {
      const uint32_t idesc = tc::idesc_f16(MODE == 2 ? 1 : 0, 128, 32);
      const int pa1[6] = {0, 1, 0, 1, 0, 2};
      const int pb1[6] = {0, 0, 1, 1, 2, 0};
      const int pa0[3] = {0, 1, 0};
      const int pb0[3] = {0, 0, 1};
      const int npair = (MODE == 1) ? 3 : 6;
      int n = 0;
      for (int p = 0; p < npair; p++) {
        const int ia = (MODE == 1) ? pa0[p] : pa1[p];
        const int ib = (MODE == 1) ? pb0[p] : pb1[p];
#pragma unroll
        for (int ks = 0; ks < 2; ks++) {
          const uint64_t ad =
              tc::smem_desc(tc::smem_u32(sa) + ia * A_PLANE + ks * 256, 128, 512);
          const uint64_t bd =
              tc::smem_desc(tc::smem_u32(sb) + ib * B_PLANE + ks * 256, 128, 512);
          tc::mma_f16(tcol, ad, bd, idesc, n > 0 ? 1u : 0u);
          n++;
        }
      }
      tc::mma_commit(mbar);
    }
    if (!tc::mbar_wait_bounded(mbar, phase, WAIT_LIMIT)) atomicExch(&g_tc_status, 1);
    phase ^= 1u;
    tc::fence_after_sync();
    float o[32];
    tc::tmem_ld32(tcol + ((uint32_t)(32 * ((threadIdx.x >> 5) & 3)) << 16), o);
#pragma unroll
    for (int k = 0; k < 16; k++) v[k] = make_float2(o[k] * us, o[16 + k] * us);
    (void)NP;
    tc::fence_before_sync();
    wg_bar(bar_id);
    tc::fence_after_sync();
  }
};

// Shared-memory map of a TC kernel: [exchange][B planes][A planes per
// warpgroup][mbarriers, TMEM slot]
template <int XCH_BYTES, int MODE, int NWG>
struct TcSmem {
  static constexpr int NP = TcTerms<MODE>::NP;
  static constexpr int OFF_B = align1k(XCH_BYTES);
  static constexpr int OFF_A = OFF_B + align1k(NP * B_PLANE);
  static constexpr int OFF_BAR = OFF_A + NWG * NP * A_PLANE;
  static constexpr int BYTES = OFF_BAR + 64;
  static constexpr uint32_t TMEM_COLS = (NWG <= 1) ? 32 : (NWG <= 2 ? 64 : 128);
};

// CTA set-up shared by both kernels: B planes, barriers, TMEM.
template <int MODE, int NWG, class SM>
__device__ __forceinline__ uint32_t tc_setup(uint8_t *sm8, int tid) {
  constexpr int NP = SM::NP;
  for (int i = tid; i < 32 * 32; i += NWG * 128) {
    const int n = i >> 5, k = i & 31;
    store_terms<MODE>(sm8 + SM::OFF_B, B_PLANE, tc::core_off(n, k, 32), g_tc_bmat[i]);
  }
  uint64_t *mbar = (uint64_t *)(sm8 + SM::OFF_BAR);
  uint32_t *slot = (uint32_t *)(sm8 + SM::OFF_BAR + 32);
  if (tid < NWG) tc::mbar_init(&mbar[tid], 1);
  if ((tid >> 5) == 0) {
    tc::tmem_alloc(slot, SM::TMEM_COLS);
    tc::tmem_relinquish();
  }
  (void)NP;
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  return *slot;
}

template <int MODE, class SM>
__device__ __forceinline__ void tc_teardown(uint32_t taddr, int tid) {
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if ((tid >> 5) == 0) tc::tmem_dealloc(taddr, SM::TMEM_COLS);
}

template <int L>
struct RowsTc {
  using C = Stock<L, 16>;
  static constexpr int THREADS = 256, NWG = 2;
  static constexpr int F = THREADS / C::T;
  static constexpr int XCH = F * L * (int)sizeof(float2);
};

template <int L, int MODE, bool INV>
__global__ void __launch_bounds__(256) k_rows_tc(const RowsArgs a) {
  using K = RowsTc<L>;
  using C = typename K::C;
  using SM = TcSmem<K::XCH, MODE, K::NWG>;
  constexpr int T = C::T, E = C::E;
  extern __shared__ __align__(1024) uint8_t sm8[];
  const int tid = threadIdx.x;
  const uint32_t taddr = tc_setup<MODE, K::NWG, SM>(sm8, tid);
  const int wg = tid >> 7;
  TcRadix16<MODE> r16{sm8 + SM::OFF_A + wg * SM::NP * A_PLANE, sm8 + SM::OFF_B,
                      (uint64_t *)(sm8 + SM::OFF_BAR) + wg, taddr + 32u * wg, 0u,
                      tid & 127, 1 + wg};

  const int fl = tid / T;
  const int t = tid - fl * T;
  const long long row = (long long)blockIdx.x * K::F + fl;
  const bool ok = row < a.nrows;
  const float2 *src = a.in + row * L;
  float2 v[E];
#pragma unroll
  for (int q = 0; q < E; q++) {
    const float2 x = ok ? src[in_index<C>(t, q)] : make_float2(0.f, 0.f);
    v[q] = INV ? cswap(x) : x;
  }
  float2 *mysm = (float2 *)sm8 + fl * L;
  stockham<C>(v, t, [mysm](int i) -> float2 & { return mysm[swz(i)]; }, a.tw, r16);
  if (ok) {
    float2 *dst = a.out + row * L;
#pragma unroll
    for (int q = 0; q < E; q++) {
      float2 x = v[q];
      if (a.scale != 1.0f) x = cscale(x, a.scale);
      dst[out_index<C>(t, q)] = INV ? cswap(x) : x;
    }
  }
  tc_teardown<MODE, SM>(taddr, tid);
}

template <int L>
struct ColsTc {
  using C = Stock<L, 16>;
  static constexpr int THREADS = 256, NWG = 2;
  static constexpr int W = THREADS / C::T;
  static constexpr int WP = W + 1;
  static constexpr int XCH = L * WP * (int)sizeof(float2);
};

template <int L, int MODE, bool INV>
__global__ void __launch_bounds__(256) k_cols_tc(const ColsArgs a) {
  using K = ColsTc<L>;
  using C = typename K::C;
  using SM = TcSmem<K::XCH, MODE, K::NWG>;
  constexpr int E = C::E, W = K::W, WP = K::WP;
  extern __shared__ __align__(1024) uint8_t sm8[];
  const int tid = threadIdx.x;
  const uint32_t taddr = tc_setup<MODE, K::NWG, SM>(sm8, tid);
  const int wg = tid >> 7;
  TcRadix16<MODE> r16{sm8 + SM::OFF_A + wg * SM::NP * A_PLANE, sm8 + SM::OFF_B,
                      (uint64_t *)(sm8 + SM::OFF_BAR) + wg, taddr + 32u * wg, 0u,
                      tid & 127, 1 + wg};

  const int t = tid / W;
  const int fl = tid - t * W;
  const long long col = (long long)blockIdx.x * W + fl;
  const bool ok = col < a.ncols;
  const long long o = col / a.inner;
  const long long c = col - o * a.inner;
  const long long base = o * (long long)L * a.inner + c;
  float2 v[E];
#pragma unroll
  for (int q = 0; q < E; q++) {
    const float2 x = ok ? a.in[base + (long long)in_index<C>(t, q) * a.inner]
                        : make_float2(0.f, 0.f);
    v[q] = INV ? cswap(x) : x;
  }
  float2 *xs = (float2 *)sm8;
  stockham<C>(v, t, [xs, fl](int i) -> float2 & { return xs[i * WP + fl]; }, a.tw,
              r16);
  if (ok) {
#pragma unroll
    for (int q = 0; q < E; q++) {
      float2 x = v[q];
      if (a.scale != 1.0f) x = cscale(x, a.scale);
      a.out[base + (long long)out_index<C>(t, q) * a.inner] = INV ? cswap(x) : x;
    }
  }
  tc_teardown<MODE, SM>(taddr, tid);
}

// ------------------------------------------------------------ dispatch
namespace {
struct TcEntry {
  int log_l;
  void (*rows[2][2])(const RowsArgs);  // [mode-1][inverse]
  void (*cols[2][2])(const ColsArgs);
  int rows_smem[2], cols_smem[2];
  int rows_f, cols_w;
};
#define TCE(L)                                                                  \
  {ilog2c(L),                                                                   \
   {{k_rows_tc<L, 1, false>, k_rows_tc<L, 1, true>},                            \
    {k_rows_tc<L, 2, false>, k_rows_tc<L, 2, true>}},                           \
   {{k_cols_tc<L, 1, false>, k_cols_tc<L, 1, true>},                            \
    {k_cols_tc<L, 2, false>, k_cols_tc<L, 2, true>}},                           \
   {TcSmem<RowsTc<L>::XCH, 1, 2>::BYTES, TcSmem<RowsTc<L>::XCH, 2, 2>::BYTES}, \
   {TcSmem<ColsTc<L>::XCH, 1, 2>::BYTES, TcSmem<ColsTc<L>::XCH, 2, 2>::BYTES}, \
   RowsTc<L>::F, ColsTc<L>::W}
const TcEntry kTc[] = {TCE(256), TCE(512)};
bool g_tc_ready = false;

const TcEntry *find_tc(int log_l) {
  for (const TcEntry &e : kTc)
    if (e.log_l == log_l) return &e;
  return nullptr;
}
}  // namespace

cudaError_t tc_kernels_init() {
  if (g_tc_ready) return cudaSuccess;
  float b[32 * 32];
  for (int j = 0; j < 16; j++)
    for (int n = 0; n < 16; n++) {
      double s, c;
      sincos(-2.0 * M_PI * ((double)((j * n) % 16) / 16.0), &s, &c);
      b[j * 32 + n] = (float)c;             // re out <- re in
      b[j * 32 + 16 + n] = (float)(-s);     // re out <- im in
      b[(16 + j) * 32 + n] = (float)s;      // im out <- re in
      b[(16 + j) * 32 + 16 + n] = (float)c; // im out <- im in
    }
  cudaError_t e = cudaMemcpyToSymbol(g_tc_bmat, b, sizeof(b));
  if (e != cudaSuccess) return e;
  const int zero = 0;
  e = cudaMemcpyToSymbol(g_tc_status, &zero, sizeof(int));
  if (e != cudaSuccess) return e;
  for (const TcEntry &t : kTc)
    for (int m = 0; m < 2; m++)
      for (int d = 0; d < 2; d++) {
        e = cudaFuncSetAttribute((const void *)t.rows[m][d],
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 t.rows_smem[m]);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute((const void *)t.cols[m][d],
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 t.cols_smem[m]);
        if (e != cudaSuccess) return e;
      }
  g_tc_ready = true;
  return cudaSuccess;
}

bool tc_available(int log_l) { return find_tc(log_l) != nullptr; }

cudaError_t launch_rows_tc(int log_l, int mode, const RowsArgs &a, cudaStream_t s) {
  const TcEntry *t = find_tc(log_l);
  if (!g_tc_ready || !t || mode < 1 || mode > 2) return cudaErrorInvalidValue;
  const long long grid = (a.nrows + t->rows_f - 1) / t->rows_f;
  if (grid <= 0 || grid > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  t->rows[mode - 1][a.swap_io ? 1 : 0]<<<(unsigned)grid, 256, t->rows_smem[mode - 1],
                                         s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_cols_tc(int log_l, int mode, const ColsArgs &a, cudaStream_t s) {
  const TcEntry *t = find_tc(log_l);
  if (!g_tc_ready || !t || mode < 1 || mode > 2) return cudaErrorInvalidValue;
  if (a.out_mode != 0 || a.tw4_lo != nullptr) return cudaErrorInvalidValue;
  const long long grid = (a.ncols + t->cols_w - 1) / t->cols_w;
  if (grid <= 0 || grid > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  t->cols[mode - 1][a.swap_io ? 1 : 0]<<<(unsigned)grid, 256, t->cols_smem[mode - 1],
                                         s>>>(a);
  return cudaGetLastError();
}

cudaError_t tc_expire_wait(unsigned polls) {
  k_tc_expire<<<1, 32>>>(polls);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? cudaDeviceSynchronize() : e;
}

int tc_status_and_clear() {
  int st = 0;
  const int zero = 0;
  if (cudaMemcpyFromSymbol(&st, g_tc_status, sizeof(int)) != cudaSuccess) return -1;
  cudaMemcpyToSymbol(g_tc_status, &zero, sizeof(int));
  return st;
}

}  // namespace fftgb
