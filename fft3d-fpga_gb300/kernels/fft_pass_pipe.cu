// fft_pass_pipe.cu - persistent, software-pipelined form of the strided-axis
// pass k_cols (fft_pass.cu): FFTs of length L along a strided axis for W
// adjacent columns per tile, in place.
//
// k_cols loads a tile, computes and stores it, one tile per CTA.
// k_cols_pipe keeps 512-thread CTAs resident (two per SM) and walks tiles
// blockIdx.x, blockIdx.x + gridDim.x, ...; the next tile is fetched with
// cp.async (16 bytes, L2 only) into the shared-memory tile as soon as the
// transform has read its last-stage inputs, so the fetch overlaps the last
// stage and the stores.  Tile rows are padded to W + 2 points so that every
// row starts on a 16-byte boundary; with W >= 16 one row spans all 32 banks
// and the padding costs no extra wavefronts.  A tile never straddles two
// outer blocks (inner % W == 0), the columns a tile stores are the ones it
// loaded, and tiles are disjoint, so prefetching tile i+1 while tile i is
// stored never reads what tile i writes.
#include "fft_core.cuh"
#include "fft_pass.cuh"

namespace fftgb {

template <int L>
struct ColsPipeCfg {
  static constexpr int E = (L <= 64) ? 8 : 16;
  using C = Stock<L, E>;
  static constexpr int THREADS = 512;
  static constexpr int W = THREADS / C::T;   // columns per tile
  static constexpr int WP = W + 2;           // padded row (16-byte aligned)
  static constexpr int SMEM = L * WP * (int)sizeof(float2);
  static constexpr int XH = W / 2;           // 16-byte copies per tile row
  static constexpr int COPIES = L * XH / THREADS;
  static_assert(W % 2 == 0 && (L * XH) % THREADS == 0, "copy split");
};

template <int L, bool INV>
__global__ void __launch_bounds__(512, 2) k_cols_pipe(const ColsArgs a, long long ntiles) {
  using K = ColsPipeCfg<L>;
  using C = typename K::C;
  constexpr int E = K::E, W = K::W, WP = K::WP, XH = K::XH;
  extern __shared__ float2 tile[];
  const int tid = threadIdx.x;
  const int t = tid / W;
  const int fl = tid - t * W;

  auto origin = [&](long long tl) -> long long {  // point (k = 0) of column tl*W
    const long long col0 = tl * W;
    const long long o = col0 / a.inner;
    return o * (long long)L * a.inner + (col0 - o * a.inner);
  };
  auto issue = [&](long long tl) {
    const float2 *src = a.in + origin(tl);
#pragma unroll
    for (int i = 0; i < K::COPIES; i++) {
      const int c = tid + i * K::THREADS;
      const int row = c / XH;
      const int xp = c - row * XH;
      cp_async16(&tile[row * WP + 2 * xp], src + (long long)row * a.inner + 2 * xp);
    }
    cp_async_commit();
  };

  long long tl = blockIdx.x;
  if (tl < ntiles) issue(tl);
  for (; tl < ntiles; tl += gridDim.x) {
    cp_async_wait_all();
    __syncthreads();  // tile tl is in shared memory
    float2 v[E];
#pragma unroll
    for (int q = 0; q < E; q++) {
      const float2 x = tile[in_index<C>(t, q) * WP + fl];
      v[q] = INV ? cswap(x) : x;
    }
    __syncthreads();
    const long long next = tl + gridDim.x;
    auto hook = [&]() {
      __syncthreads();  // every thread has read its last-stage inputs
      if (next < ntiles) issue(next);
    };
    stockham_h<C>(v, t, [fl](int i) -> float2 & {
      extern __shared__ float2 tile_[];
      return tile_[i * WP + fl];
    }, a.tw, hook);
    const long long col = tl * W + fl;
    if (a.tw4_lo != nullptr) {
      const long long c = col % a.inner;
      tw4_mul<C, true>(v, t, c, a.tw4_lo, a.tw4_hi, a.tw4_bits);
    }
    float2 *dst = a.out + origin(tl) + fl;
#pragma unroll
    for (int q = 0; q < E; q++) {
      float2 x = v[q];
      if (a.scale != 1.0f) x = cscale(x, a.scale);
      dst[(long long)out_index<C>(t, q) * a.inner] = INV ? cswap(x) : x;
    }
  }
}

namespace {
struct PipeCols {
  int log_l;
  void (*fn[2])(const ColsArgs, long long);
  int smem, w, e;
  int grid;  // resident CTAs (occupancy x SMs)
};
#define CP(L)                                                               \
  {ilog2c(L), {k_cols_pipe<L, false>, k_cols_pipe<L, true>},                \
   ColsPipeCfg<L>::SMEM, ColsPipeCfg<L>::W, ColsPipeCfg<L>::E, 0}
PipeCols kColsPipe[] = {CP(64), CP(128), CP(256), CP(512)};
bool g_cp_ready = false;

const PipeCols *find(int log_l) {
  for (const PipeCols &p : kColsPipe)
    if (p.log_l == log_l) return &p;
  return nullptr;
}
}  // namespace

cudaError_t cols_pipe_init() {
  if (g_cp_ready) return cudaSuccess;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  for (PipeCols &p : kColsPipe) {
    for (int d = 0; d < 2; d++) {
      e = cudaFuncSetAttribute((const void *)p.fn[d],
                               cudaFuncAttributeMaxDynamicSharedMemorySize, p.smem);
      if (e != cudaSuccess) return e;
    }
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, p.fn[0], 512, p.smem);
    if (e != cudaSuccess) return e;
    p.grid = (occ > 0 ? occ : 1) * sms;
  }
  g_cp_ready = true;
  return cudaSuccess;
}

int cols_pipe_e(int log_l) {
  const PipeCols *p = find(log_l);
  return p ? p->e : 0;
}

bool cols_pipe_supported(int log_l, long long ncols, long long inner) {
  const PipeCols *p = find(log_l);
  return p && inner % p->w == 0 && ncols % p->w == 0 && ncols > 0;
}

cudaError_t launch_cols_pipe(int log_l, const ColsArgs &a, cudaStream_t s) {
  const PipeCols *p = find(log_l);
  if (!g_cp_ready || !p || a.out_mode != 0 || !cols_pipe_supported(log_l, a.ncols, a.inner))
    return cudaErrorInvalidValue;
  if (((uintptr_t)a.in & 15) || ((uintptr_t)a.out & 15)) return cudaErrorMisalignedAddress;
  const long long ntiles = a.ncols / p->w;
  const int grid = ntiles < p->grid ? (int)ntiles : p->grid;
  p->fn[a.swap_io ? 1 : 0]<<<grid, 512, p->smem, s>>>(a, ntiles);
  return cudaGetLastError();
}

}  // namespace fftgb
