// fft_ragged.cu - one persistent launch over a work list of row and column
// tiles: a ragged batch of 3D grids (independent power-of-two shapes), or a
// batch of uniform transforms whose passes run chunk by chunk so that each
// chunk's intermediate stays in L2 between its passes.
//
// The host builds the work list (shim/ragged.cu): the tiles of every pass of
// every unit, pass p of chunk c emitted at step c + p.  Persistent CTAs
// claim items in list order from an atomic counter.  An item of pass p of a
// unit first waits until all tiles of pass p-1 of that unit are done; those
// were emitted earlier in the list, and every item is claimed only by a
// running CTA (each CTA claims its next item while it works on the current
// one), so everything an item waits for is being processed or queued behind
// an earlier item of a running CTA, and the wait ends.  It is nevertheless
// bounded: after ~2^26 polls the CTA
// records a timeout in the status word and goes on (results are then
// invalid, the GPU never hangs).  Data written by other SMs is read with
// ld.global.cg (L2), not through L1.
#include "fft_core.cuh"
#include "fft_ragged.cuh"

namespace fftgb {

namespace {
constexpr int RG_THREADS = 512;
constexpr unsigned RG_SPIN_LIMIT = 1u << 26;

template <int L>
struct RgGeo {
  using C = Cfg<L>;
  static constexpr int F = RG_THREADS / C::T;  // rows per row tile
  static constexpr int W = RG_THREADS / C::T;  // columns per column tile
  static constexpr int SMEM_ROWS = F * L * (int)sizeof(float2);
  static constexpr int SMEM_COLS = L * (W + 1) * (int)sizeof(float2);
};
}  // namespace

template <int L, bool INV>
__device__ __forceinline__ void rg_rows(const RgArgs &a, const RgItem &it,
                                        float2 *smem) {
  using C = Cfg<L>;
  constexpr int T = C::T, E = C::E;
  const int tid = threadIdx.x;
  const int fl = tid / T;
  const int t = tid - fl * T;
  const long long row = it.first + fl;
  const bool ok = row < it.count;
  const float2 *src = (it.src_in ? a.in : a.out) + it.base + row * L;
  float2 *dst = a.out + it.base + row * L;
  float2 v[E];
#pragma unroll
  for (int q = 0; q < E; q++) {
    const float2 x = ok ? __ldcg(&src[in_index<C>(t, q)]) : make_float2(0.f, 0.f);
    v[q] = INV ? cswap(x) : x;
  }
  float2 *row_sm = smem + fl * L;
  stockham_row<C, RgGeo<L>::F>(v, t, [row_sm](int i) -> float2 & { return row_sm[swz(i)]; },
                               a.tw[C::LOG], fl);
  if (it.scale) {
#pragma unroll
    for (int q = 0; q < E; q++) v[q] = cscale(v[q], a.scale);
  }
  if (ok) {
#pragma unroll
    for (int q = 0; q < E; q++) dst[out_index<C>(t, q)] = INV ? cswap(v[q]) : v[q];
  }
}

template <int L, bool INV>
__device__ __forceinline__ void rg_cols(const RgArgs &a, const RgItem &it,
                                        float2 *smem) {
  using C = Cfg<L>;
  constexpr int E = C::E, W = RgGeo<L>::W, WP = W + 1;
  const int tid = threadIdx.x;
  const int t = tid / W;
  const int fl = tid - t * W;
  const long long col = it.first + fl;
  const bool ok = col < it.count;
  // per-grid numbers fit 32 bits: 32-bit division
  const unsigned oq = (unsigned)col / (unsigned)it.inner;
  const long long o = oq;
  const long long c = (long long)((unsigned)col - oq * (unsigned)it.inner);
  const long long base = it.base + o * (long long)L * it.inner + c;
  const float2 *src = it.src_in ? a.in : a.out;
  float2 v[E];
#pragma unroll
  for (int q = 0; q < E; q++) {
    const float2 x = ok ? __ldcg(&src[base + (long long)in_index<C>(t, q) * it.inner])
                        : make_float2(0.f, 0.f);
    v[q] = INV ? cswap(x) : x;
  }
  stockham<C>(v, t, [smem, fl](int i) -> float2 & { return smem[i * WP + fl]; },
              a.tw[C::LOG]);
  if (it.scale) {
#pragma unroll
    for (int q = 0; q < E; q++) v[q] = cscale(v[q], a.scale);
  }
  if (ok) {
#pragma unroll
    for (int q = 0; q < E; q++)
      a.out[base + (long long)out_index<C>(t, q) * it.inner] =
          INV ? cswap(v[q]) : v[q];
  }
}

constexpr int RG_TILE = RG_THREADS * 16;

// kind 3: P = RG_TILE / (NX*NJ) planes, rows y = R*j + r of each, x FFT,
// NJ-point y FFT, twiddle W_ny^(r*k1), rows r*NJ + k1 stored.
template <int NX, int NJ, bool INV>
__device__ __forceinline__ void rg_xy(const RgArgs &a, const RgItem &it, float2 *smem) {
  using CX = Stock<NX, 16>;
  using CJ = Stock<NJ, 16>;
  constexpr int E = 16;
  constexpr int P = RG_TILE / (NX * NJ);
  static_assert(P >= 1 && P * NJ * NX == RG_TILE, "tile");
  const int tid = threadIdx.x;
  const long long ny = it.inner;
  const int R = (int)(ny / NJ);
  const unsigned pq = (unsigned)it.first / (unsigned)R;  // 32-bit: per-grid tile numbers
  const long long p0 = (long long)pq * P;
  const int r = (int)((unsigned)it.first - pq * (unsigned)R);
  {
    const int rr = tid / CX::T;  // row of the tile: plane rr / NJ, j = rr % NJ
    const int t = tid - rr * CX::T;
    const int pl = rr / NJ, j = rr - pl * NJ;
    const float2 *src = (it.src_in ? a.in : a.out) + it.base +
                        ((p0 + pl) * ny + (long long)R * j + r) * NX;
    float2 v[E];
#pragma unroll
    for (int q = 0; q < E; q++) {
      const float2 x = __ldcg(&src[in_index<CX>(t, q)]);
      v[q] = INV ? cswap(x) : x;
    }
    float2 *row = smem + rr * NX;
    stockham_row<CX, P * NJ>(v, t, [row](int i) -> float2 & { return row[swz(i)]; },
                             a.tw16[CX::LOG], rr);
    row_sync<CX, P * NJ>(rr);
#pragma unroll
    for (int q = 0; q < E; q++) row[out_index<CX>(t, q)] = v[q];
  }
  __syncthreads();
  constexpr int TJ = CJ::T;
  const int pl = tid / (NX * TJ);
  const int rem = tid - pl * (NX * TJ);
  const int k = rem % NX;
  const int t = rem / NX;
  float2 *pt = smem + pl * NJ * NX;
  float2 v[E];
#pragma unroll
  for (int q = 0; q < E; q++) v[q] = pt[in_index<CJ>(t, q) * NX + k];
  __syncthreads();
  stockham<CJ>(v, t, [pt, k](int i) -> float2 & { return pt[i * NX + k]; },
               a.tw16[CJ::LOG]);
  const float2 *twy = a.tww[__ffsll(ny) - 1];
  float2 *dst = a.out + it.base + ((p0 + pl) * ny + (long long)r * NJ) * NX + k;
#pragma unroll
  for (int q = 0; q < E; q++) {
    const int k1 = out_index<CJ>(t, q);
    float2 x = v[q];
    if (R > 1) x = cmul(x, __ldg(&twy[r * k1]));
    if (it.scale) x = cscale(x, a.scale);
    dst[(long long)k1 * NX] = INV ? cswap(x) : x;
  }
}

// kind 4: radix-R over the residue rows r*nj + k1 of X = RG_TILE/(R*NZ)
// columns of every plane, then the z FFT; in place.
template <int NZ, int R, bool INV>
__device__ __forceinline__ void rg_rz(const RgArgs &a, const RgItem &it, float2 *smem) {
  constexpr int X = RG_TILE / (R * NZ);
  using CZ = Stock<NZ, 16>;
  constexpr int E = 16;
  constexpr int KS = NZ * X + (X < 16 ? X : 0);  // residue block stride (banks)
  static_assert(R * NZ * X == RG_TILE && E % R == 0, "tile");
  const int tid = threadIdx.x;
  const long long nx = it.inner;
  // per-grid numbers fit 32 bits: 32-bit divisions
  const unsigned xblocks = (unsigned)nx / X;
  const long long nj = (unsigned)it.count / xblocks;
  const long long plane = nj * R * nx;
  const unsigned kq = (unsigned)it.first / xblocks;
  const long long xb = (unsigned)it.first - kq * xblocks;
  const long long k1 = kq;
  float2 *g = a.out + it.base + k1 * nx + xb * X;
  const int x = tid % X;
  {
    constexpr int ITEMS = E / R;
    constexpr int ZSTEP = RG_THREADS / X;
    const int z0 = tid / X;
#pragma unroll
    for (int m = 0; m < ITEMS; m++) {
      const int z = z0 + m * ZSTEP;
      float2 u[R];
#pragma unroll
      for (int rr = 0; rr < R; rr++) {
        const float2 w = __ldcg(&g[z * plane + rr * nj * nx + x]);
        u[rr] = INV ? cswap(w) : w;
      }
      dft<R>(u);
#pragma unroll
      for (int k2 = 0; k2 < R; k2++) smem[k2 * KS + z * X + x] = u[k2];
    }
  }
  __syncthreads();
  const int k2 = (tid / X) % R;
  const int t = tid / (X * R);
  float2 v[E];
#pragma unroll
  for (int q = 0; q < E; q++) v[q] = smem[k2 * KS + in_index<CZ>(t, q) * X + x];
  __syncthreads();
  stockham<CZ>(v, t, [smem, k2, x](int i) -> float2 & { return smem[k2 * KS + i * X + x]; },
               a.tw16[CZ::LOG]);
  float2 *d = g + k2 * nj * nx;
#pragma unroll
  for (int q = 0; q < E; q++) {
    float2 w = v[q];
    if (it.scale) w = cscale(w, a.scale);
    d[out_index<CZ>(t, q) * plane + x] = INV ? cswap(w) : w;
  }
}

#define RG_XY(NX, NJ) \
  case ilog2c(NX) * 16 + ilog2c(NJ): rg_xy<NX, NJ, INV>(a, it, smem); break;
#define RG_RZ(NZ, R) \
  case ilog2c(NZ) * 16 + ilog2c(R): rg_rz<NZ, R, INV>(a, it, smem); break;

template <bool INV>
__device__ __forceinline__ void rg_fused(const RgArgs &a, const RgItem &it, float2 *smem) {
  const int key = it.log_l * 16 + (__ffs(it.aux) - 1);
  if (it.kind == 3) {
    switch (key) {
      RG_XY(256, 32) RG_XY(128, 32) RG_XY(128, 64) RG_XY(64, 32) RG_XY(64, 64)
      RG_XY(64, 128) RG_XY(32, 32) RG_XY(32, 64) RG_XY(32, 128) RG_XY(32, 256)
      default: break;
    }
  } else {
    switch (key) {
      RG_RZ(256, 2) RG_RZ(256, 4) RG_RZ(256, 8) RG_RZ(128, 2) RG_RZ(128, 4)
      RG_RZ(128, 8) RG_RZ(64, 2) RG_RZ(64, 4) RG_RZ(64, 8) RG_RZ(32, 2)
      RG_RZ(32, 4) RG_RZ(32, 8)
      default: break;
    }
  }
}

// Waits until counter *ctr reaches `target`, polling with a short sleep and
// giving up after `limit` polls; a wait that gives up sets *status.
__device__ __forceinline__ void rg_wait_count(const int *ctr, int target, int *status,
                                              unsigned limit) {
  unsigned spins = 0;
  while (*((volatile const int *)ctr) < target) {
    __nanosleep(128);
    if (++spins > limit) {
      atomicExch(status, 1);
      break;
    }
  }
  __threadfence();
}

// The dependency wait's give-up path on demand: one thread waits for a
// counter to reach INT_MAX, which nothing does, and gives up after `polls`.
__global__ void k_ragged_expire(const int *ctr, int *status, unsigned polls) {
  if (threadIdx.x == 0) rg_wait_count(ctr, 0x7fffffff, status, polls);
}

template <bool INV>
__global__ void __launch_bounds__(RG_THREADS, 2) k_ragged(const RgArgs a) {
  extern __shared__ float2 smem[];
  __shared__ int s_item;
  const int tid = threadIdx.x;
  if (tid == 0) s_item = atomicAdd(a.counter, 1);
  __syncthreads();
  int next = 0;  // thread 0: the item claimed ahead of this one's end
  while (true) {
    const int i = s_item;
    if (i >= a.nitems) break;
    // claim the following item now, so that the atomic's round trip overlaps
    // this item's work (a CTA holds at most two claims, taken in list
    // order: the smallest unfinished item is always some CTA's current one,
    // so the dependency waits still end)
    if (tid == 0) next = atomicAdd(a.counter, 1);
    const RgItem it = a.items[i];
    if (it.dep >= 0) {
      if (tid == 0) rg_wait_count(&a.done[it.dep], it.dep_target, a.status, RG_SPIN_LIMIT);
      __syncthreads();
    }
    if (it.kind >= 3) rg_fused<INV>(a, it, smem);
    else switch (it.kind * 16 + it.log_l) {
      case 0 * 16 + 4: rg_rows<16, INV>(a, it, smem); break;
      case 0 * 16 + 5: rg_rows<32, INV>(a, it, smem); break;
      case 0 * 16 + 6: rg_rows<64, INV>(a, it, smem); break;
      case 0 * 16 + 7: rg_rows<128, INV>(a, it, smem); break;
      case 0 * 16 + 8: rg_rows<256, INV>(a, it, smem); break;
      case 0 * 16 + 9: rg_rows<512, INV>(a, it, smem); break;
      case 0 * 16 + 10: rg_rows<1024, INV>(a, it, smem); break;
      case 1 * 16 + 4: rg_cols<16, INV>(a, it, smem); break;
      case 1 * 16 + 5: rg_cols<32, INV>(a, it, smem); break;
      case 1 * 16 + 6: rg_cols<64, INV>(a, it, smem); break;
      case 1 * 16 + 7: rg_cols<128, INV>(a, it, smem); break;
      case 1 * 16 + 8: rg_cols<256, INV>(a, it, smem); break;
      case 1 * 16 + 9: rg_cols<512, INV>(a, it, smem); break;
      case 1 * 16 + 10: rg_cols<1024, INV>(a, it, smem); break;
      default: break;
    }
    // Every thread's stores of this item precede the barrier; thread 0's
    // device-scope fence after it is cumulative over them, so the done count
    // is published after the item's whole output (the release pattern of a
    // grid barrier).  The barrier also frees shared memory and s_item for
    // the next item.
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      atomicAdd(&a.done[it.done_id], 1);
      s_item = next;
    }
    __syncthreads();
  }
}

namespace {
constexpr int kMaxSmem() {
  int m = 0;
  const int r[] = {RgGeo<16>::SMEM_ROWS, RgGeo<32>::SMEM_ROWS, RgGeo<64>::SMEM_ROWS,
                   RgGeo<128>::SMEM_ROWS, RgGeo<256>::SMEM_ROWS, RgGeo<512>::SMEM_ROWS,
                   RgGeo<1024>::SMEM_ROWS,
                   RgGeo<16>::SMEM_COLS, RgGeo<32>::SMEM_COLS, RgGeo<64>::SMEM_COLS,
                   RgGeo<128>::SMEM_COLS, RgGeo<256>::SMEM_COLS, RgGeo<512>::SMEM_COLS,
                   RgGeo<1024>::SMEM_COLS};
  for (int v : r) m = v > m ? v : m;
  return m;
}
constexpr int RG_SMEM = kMaxSmem();
bool g_rg_ready = false;
int g_rg_grid = 0;
}  // namespace

bool ragged_axis_supported(int log_l) { return log_l >= 4 && log_l <= 10; }

bool ragged_fused_supported(int kind, int log_l, int aux) {
  if (kind == 3) {  // (NX, NJ) with NX * NJ <= 8192
    const int l = log_l, j = aux > 0 ? __builtin_ctz((unsigned)aux) : 0;
    return aux > 0 && (aux & (aux - 1)) == 0 && l >= 5 && l <= 8 && j >= 5 &&
           l + j <= 13 && (l == 5 ? j <= 8 : true);
  }
  if (kind == 4)  // (NZ, R): NZ 32..256, R 2..8
    return log_l >= 5 && log_l <= 8 && (aux == 2 || aux == 4 || aux == 8);
  return false;
}

int ragged_fused_tile_points() { return RG_TILE; }

int ragged_rows_per_tile(int log_l) {
  switch (log_l) {
    case 4: return RgGeo<16>::F;
    case 5: return RgGeo<32>::F;
    case 6: return RgGeo<64>::F;
    case 7: return RgGeo<128>::F;
    case 8: return RgGeo<256>::F;
    case 9: return RgGeo<512>::F;
    case 10: return RgGeo<1024>::F;
  }
  return 0;
}

int ragged_cols_per_tile(int log_l) { return ragged_rows_per_tile(log_l); }

cudaError_t ragged_init(int device) {
  if (g_rg_ready) return cudaSuccess;
  cudaError_t e;
  for (int d = 0; d < 2; d++) {
    e = cudaFuncSetAttribute(d ? (const void *)k_ragged<true> : (const void *)k_ragged<false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, RG_SMEM);
    if (e != cudaSuccess) return e;
  }
  int occ = 0, sms = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_ragged<false>, RG_THREADS,
                                                    RG_SMEM);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return e;
  g_rg_grid = (occ > 0 ? occ : 1) * sms;
  g_rg_ready = true;
  return cudaSuccess;
}

cudaError_t launch_ragged(const RgArgs &a, int inverse, cudaStream_t s) {
  if (!g_rg_ready) return cudaErrorInvalidValue;
  const int grid = a.nitems < g_rg_grid ? a.nitems : g_rg_grid;
  if (grid <= 0) return cudaSuccess;
  if (inverse)
    k_ragged<true><<<grid, RG_THREADS, RG_SMEM, s>>>(a);
  else
    k_ragged<false><<<grid, RG_THREADS, RG_SMEM, s>>>(a);
  return cudaGetLastError();
}

cudaError_t ragged_expire_wait(const int *ctr, int *status, unsigned polls) {
  k_ragged_expire<<<1, 32>>>(ctr, status, polls);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? cudaDeviceSynchronize() : e;
}

}  // namespace fftgb
