// fft_pass_tma.cu - persistent form of the strided-axis pass k_cols
// (fft_pass.cu) whose tiles arrive by TMA tensor copies into alternating
// shared-memory buffers (and, for 512-point columns, leave by TMA tensor
// stores from the same buffers): FFTs of length L along a strided axis for W
// adjacent columns per tile, in place or out of place (same layout), with
// the four-step twiddle on the outputs as k_cols applies it.  The transposed
// store (out_mode 1) and the twiddle on the inputs (tw_in) stay with k_cols:
// with tw_in this kernel measured 5-9 % slower than k_cols on GB300 (1D
// 65536 x 1024 second pass 0.206 against 0.195 ms, 2D 1024^2 x 64 column
// pass 0.188 against 0.179), whether the factors were read before or after
// the tile's wait.
//
// The data is a 3D tensor [outer][n][inner] (n < L the transform index, the
// column c < inner contiguous); a tile is the L x W block of columns
// [c0, c0 + W) of one outer block, copied as L / BR boxes {W, BR, 1} (a box
// dimension holds at most 256 elements).  One 512-thread CTA per SM walks
// tiles blockIdx.x, blockIdx.x + gridDim.x, ...: while it transforms tile i
// in buffer i % 2 (in place, exchanges included: with W >= 16 columns a
// half-warp's 64-bit accesses cover one 128-byte row run, so the unpadded
// rows are free of bank conflicts), tile i + 1 is already arriving in the
// other buffer, and tile i + 2 is requested into buffer i % 2 as soon as
// every thread has read its last-stage inputs.  With TMA stores (512-point
// columns) the outputs go back into the tile's buffer and leave by tensor
// stores, and three buffers rotate: tile i + 2 goes into the buffer of tile
// i - 1 once that tile's stores have read it.  Tiles are disjoint and a
// tile stores only the columns it loaded, so no prefetch reads what an
// earlier tile writes.  mbarrier waits are bounded (2^24 polls): on a
// timeout the kernel records it in a status word and goes on (results
// invalid, never a hang).
#include <cuda.h>

#include "fft_core.cuh"
#include "fft_pass.cuh"
#include "tc_core.cuh"

namespace fftgb {

namespace {
constexpr uint32_t CT_WAIT_LIMIT = 1u << 24;
__device__ int g_ct_status;
__global__ void k_cols_tma_expire(uint32_t polls) { tc::expire_wait(&g_ct_status, polls); }

template <int L, bool TS>
struct ColsTmaCfg {
  using C = Cfg<L>;
  static constexpr int W = (L <= 128) ? 64 : (L <= 256) ? 32 : 16;  // as k_cols
  static constexpr int THREADS = W * C::T;
  static constexpr int TILE = L * W;                 // points per tile
  static constexpr int BR = L < 256 ? L : 256;        // rows per box
  static constexpr int NB = L / BR;                   // boxes per tile
  static constexpr int NBUF = TS ? 3 : 2;
  static constexpr int SMEM = NBUF * TILE * (int)sizeof(float2) + 32;
  static_assert(THREADS == 512, "one 512-thread CTA per SM");
  static_assert(W >= 16 && (W * 8) % 16 == 0, "box rows of whole 16-byte units");
};
}  // namespace

// TW: the outputs carry the four-step twiddle (a separate instantiation, so
// that the plain pass keeps its register allocation).  TS: the outputs go
// back into the tile's buffer and out by TMA tensor stores (three buffers: a
// buffer is refilled only once its store has read it); otherwise each
// thread stores its points.
template <int L, bool INV, bool TW, bool TS>
__global__ void __launch_bounds__(512, 1)
    k_cols_tma(const ColsArgs a, const __grid_constant__ CUtensorMap tmap,
               const __grid_constant__ CUtensorMap tmap_out, long long ntiles) {
  using K = ColsTmaCfg<L, TS>;
  using C = typename K::C;
  constexpr int E = C::E, W = K::W, TILE = K::TILE, BR = K::BR, NB = K::NB, NBUF = K::NBUF;
  constexpr uint32_t TILE_BYTES = (uint32_t)(TILE * sizeof(float2));
  extern __shared__ __align__(128) float2 buf[];
  uint64_t *mbar = reinterpret_cast<uint64_t *>(buf + NBUF * TILE);
  pdl_enter();
  const int tid = threadIdx.x;
  const int t = tid / W;
  const int fl = tid - t * W;
  const long long tpo = a.inner / W;  // tiles per outer block

  auto issue = [&](long long tl, int b) {  // one thread
    const long long o = tl / tpo;
    const int c0 = (int)((tl - o * tpo) * W);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(
                     tc::smem_u32(mbar + b)), "r"(TILE_BYTES) : "memory");
    if (a.blk_lnz >= 0) {
      // y-blocked input [b][L/8][nz][8][inner]: box {W, 8, 1, BR/8, 1} at
      // (c0, 0, z, nb*BR/8, b) lands as BR rows n = 8*(n/8) + n%8 of W points
      const int z = (int)(o & ((1LL << a.blk_lnz) - 1));
      const int bb = (int)(o >> a.blk_lnz);
#pragma unroll
      for (int nb = 0; nb < NB; nb++)
        asm volatile(
            "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes "
            "[%0], [%1, {%2, %3, %4, %5, %6}], [%7];\n" ::"r"(
                tc::smem_u32(buf + b * TILE + nb * BR * W)),
            "l"(reinterpret_cast<uint64_t>(&tmap)), "r"(c0), "r"(0), "r"(z), "r"(nb * BR / 8),
            "r"(bb), "r"(tc::smem_u32(mbar + b))
            : "memory");
      return;
    }
#pragma unroll
    for (int nb = 0; nb < NB; nb++)
      asm volatile(
          "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes "
          "[%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(tc::smem_u32(buf + b * TILE + nb * BR * W)),
          "l"(reinterpret_cast<uint64_t>(&tmap)), "r"(c0), "r"(nb * BR), "r"((int)o),
          "r"(tc::smem_u32(mbar + b))
          : "memory");
  };

  if (tid == 0) {
    for (int b = 0; b < NBUF; b++) tc::mbar_init(mbar + b, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    if (blockIdx.x < ntiles) issue(blockIdx.x, 0);
    if (blockIdx.x + gridDim.x < ntiles) issue(blockIdx.x + gridDim.x, 1);
  }
  __syncthreads();  // the mbarriers are initialised before anyone waits

  bool ok = true;
  uint32_t phases = 0;  // bit b: parity of buffer b's next completion
  int b = 0;            // this tile's buffer
  for (long long tl = blockIdx.x; tl < ntiles; tl += gridDim.x) {
    float2 *tile = buf + b * TILE;
    const long long o = tl / tpo;
    const long long c = (tl - o * tpo) * W + fl;  // column within the outer block
    ok = tc::mbar_wait_bounded(mbar + b, (phases >> b) & 1u, CT_WAIT_LIMIT) && ok;
    phases ^= 1u << b;

    float2 v[E];
#pragma unroll
    for (int q = 0; q < E; q++) {
      const float2 x = tile[in_index<C>(t, q) * W + fl];
      v[q] = INV ? cswap(x) : x;
    }
    __syncthreads();  // every stage-0 input read before the in-place exchange
    stockham<C>(v, t, [tile, fl](int m) -> float2 & { return tile[m * W + fl]; }, a.tw);
    if constexpr (TS) {
      __syncthreads();  // every last-stage input read before the outputs land
      if (TW)  // W^(c*k) on the outputs k
        tw4_mul<C, true>(v, t, c, a.tw4_lo, a.tw4_hi, a.tw4_bits);
#pragma unroll
      for (int q = 0; q < E; q++) {
        float2 x = v[q];
        if (a.scale != 1.0f) x = cscale(x, a.scale);
        tile[out_index<C>(t, q) * W + fl] = INV ? cswap(x) : x;
      }
      // order the generic writes before the tensor stores that read them
      tc::fence_proxy_async();
      __syncthreads();
      if (tid == 0) {
        const int c0 = (int)((tl - o * tpo) * W);
#pragma unroll
        for (int nb = 0; nb < NB; nb++)
          asm volatile(
              "cp.async.bulk.tensor.3d.global.shared::cta.bulk_group "
              "[%0, {%1, %2, %3}], [%4];\n" ::"l"(reinterpret_cast<uint64_t>(&tmap_out)),
              "r"(c0), "r"(nb * BR), "r"((int)o), "r"(tc::smem_u32(tile + nb * BR * W))
              : "memory");
        asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
        // the previous tile's stores have read its buffer, which takes the
        // tile after next
        asm volatile("cp.async.bulk.wait_group.read 1;\n" ::: "memory");
        const long long after = tl + 2 * (long long)gridDim.x;
        if (after < ntiles) issue(after, b == 0 ? NBUF - 1 : b - 1);
      }
    } else {
      // every thread has read its last-stage inputs: order these generic
      // accesses before the tensor copy that refills this buffer
      tc::fence_proxy_async();
      __syncthreads();
      const long long after = tl + 2 * (long long)gridDim.x;
      if (tid == 0 && after < ntiles) issue(after, b);

      if (TW)  // W^(c*k) on the outputs k
        tw4_mul<C, true>(v, t, c, a.tw4_lo, a.tw4_hi, a.tw4_bits);
      float2 *dst = a.out + o * (long long)L * a.inner + c;
#pragma unroll
      for (int q = 0; q < E; q++) {
        float2 x = v[q];
        if (a.scale != 1.0f) x = cscale(x, a.scale);
        dst[(long long)out_index<C>(t, q) * a.inner] = INV ? cswap(x) : x;
      }
    }
    b = (b + 1 == NBUF) ? 0 : b + 1;
  }
  if constexpr (TS) {
    // the last stores complete before the CTA (and its shared memory) ends
    if (tid == 0) asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
  }
  if (!ok) atomicExch(&g_ct_status, 1);
}

namespace {
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion,
                                  CUtensorMapFloatOOBfill);
struct ColsTmaEntry {
  int log_l;
  // [TS][TW][INV]
  void (*fn[2][2][2])(const ColsArgs, const CUtensorMap, const CUtensorMap, long long);
  int w, br, smem[2];
  int grid[2];
};
#define CT(L)                                                                      \
  {ilog2c(L),                                                                      \
   {{{k_cols_tma<L, false, false, false>, k_cols_tma<L, true, false, false>},      \
     {k_cols_tma<L, false, true, false>, k_cols_tma<L, true, true, false>}},       \
    {{k_cols_tma<L, false, false, true>, k_cols_tma<L, true, false, true>},        \
     {k_cols_tma<L, false, true, true>, k_cols_tma<L, true, true, true>}}},        \
   ColsTmaCfg<L, false>::W, ColsTmaCfg<L, false>::BR,                              \
   {ColsTmaCfg<L, false>::SMEM, ColsTmaCfg<L, true>::SMEM}, {0, 0}}
ColsTmaEntry kColsTma[] = {CT(128), CT(256), CT(512)};
bool g_ct_ready = false;
EncodeTiledFn g_ct_encode = nullptr;

const ColsTmaEntry *find_ct(int log_l) {
  for (const ColsTmaEntry &p : kColsTma)
    if (p.log_l == log_l) return &p;
  return nullptr;
}
}  // namespace

cudaError_t cols_tma_init() {
  if (g_ct_ready) return cudaSuccess;
  void *fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                       &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess)
    fn = nullptr;
  cudaGetLastError();
  g_ct_encode = reinterpret_cast<EncodeTiledFn>(fn);
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  for (ColsTmaEntry &p : kColsTma) {
    for (int ts = 0; ts < 2; ts++) {
      for (int d = 0; d < 4; d++) {
        e = cudaFuncSetAttribute((const void *)p.fn[ts][d >> 1][d & 1],
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, p.smem[ts]);
        if (e != cudaSuccess) return e;
      }
      int occ = 0;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, p.fn[ts][0][0], 512, p.smem[ts]);
      if (e != cudaSuccess) return e;
      p.grid[ts] = (occ > 0 ? occ : 1) * sms;
    }
  }
  g_ct_ready = true;
  return cudaSuccess;
}

bool cols_tma_supported(int log_l, long long ncols, long long inner) {
  const ColsTmaEntry *p = find_ct(log_l);
  return g_ct_encode && p && inner % p->w == 0 && ncols % p->w == 0 && ncols > 0 &&
         inner < (1LL << 31) && ncols / inner < (1LL << 31);
}

cudaError_t launch_cols_tma(int log_l, const ColsArgs &a, cudaStream_t s, bool pdl) {
  const ColsTmaEntry *p = find_ct(log_l);
  if (!g_ct_ready || !p || a.out_mode != 0 || a.tw_in ||
      !cols_tma_supported(log_l, a.ncols, a.inner))
    return cudaErrorNotSupported;
  if ((uintptr_t)a.in & 15) return cudaErrorMisalignedAddress;
  const long long L = 1LL << log_l;
  const long long outer = a.ncols / a.inner;
  const cuuint64_t dims[3] = {(cuuint64_t)a.inner, (cuuint64_t)L, (cuuint64_t)outer};
  const cuuint64_t strides[2] = {(cuuint64_t)a.inner * 8, (cuuint64_t)(L * a.inner * 8)};
  const cuuint32_t box[3] = {(cuuint32_t)p->w, (cuuint32_t)p->br, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  CUtensorMap m, mo;
  if (a.blk_lnz >= 0) {
    // y-blocked input [b][L/8][nz][8][inner] as a 5D tensor
    // {inner, 8, nz, L/8, b}; boxes {W, 8, 1, BR/8, 1}
    const long long nz = 1LL << a.blk_lnz;
    if (a.tw4_lo != nullptr || L < 64 || p->br % 8 || outer % nz) return cudaErrorNotSupported;
    const cuuint64_t bd[5] = {(cuuint64_t)a.inner, 8, (cuuint64_t)nz, (cuuint64_t)(L / 8),
                              (cuuint64_t)(outer / nz)};
    const cuuint64_t bs[4] = {(cuuint64_t)a.inner * 8, (cuuint64_t)(8 * a.inner * 8),
                              (cuuint64_t)(nz * 8 * a.inner * 8),
                              (cuuint64_t)(L * nz * a.inner * 8)};
    const cuuint32_t bbox[5] = {(cuuint32_t)p->w, 8, 1, (cuuint32_t)(p->br / 8), 1};
    const cuuint32_t bestr[5] = {1, 1, 1, 1, 1};
    if (g_ct_encode(&m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 5, const_cast<float2 *>(a.in), bd, bs,
                    bbox, bestr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return cudaErrorNotSupported;
  } else if (g_ct_encode(&m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, const_cast<float2 *>(a.in),
                         dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                         CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
    return cudaErrorNotSupported;
  }
  // outputs by TMA stores for 512-point columns (rows of 16 columns, 128-byte
  // runs) when the output allows a tensor map (16-byte aligned): 512^3 y and
  // z passes 0.348 / 0.384 against 0.388 / 0.392 ms with per-thread stores,
  // 2048^2 x 16 column pass 0.178 against 0.199.  With 32 or 64 columns the
  // per-thread stores are 256-byte runs and as fast (256^2 x 1024 column
  // pass 0.165 either way; bit-reversed 65536 x 1024 first pass 0.171
  // against 0.175 with TMA stores)
  const int ts = (log_l >= 9 && ((uintptr_t)a.out & 15) == 0) ? 1 : 0;
  mo = m;  // unused without tensor stores
  if (ts && g_ct_encode(&mo, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, a.out, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return cudaErrorNotSupported;
  const long long ntiles = a.ncols / p->w;
  const int grid = ntiles < p->grid[ts] ? (int)ntiles : p->grid[ts];
  return launch_k(p->fn[ts][a.tw4_lo != nullptr ? 1 : 0][a.swap_io ? 1 : 0], dim3(grid),
                  dim3(512), p->smem[ts], s, pdl, a, m, mo, ntiles);
}

cudaError_t cols_tma_expire_wait(unsigned polls) {
  k_cols_tma_expire<<<1, 32>>>(polls);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? cudaDeviceSynchronize() : e;
}

int cols_tma_status_and_clear() {
  int st = 0;
  const int zero = 0;
  if (cudaMemcpyFromSymbol(&st, g_ct_status, sizeof(int)) != cudaSuccess) return -1;
  if (st && cudaMemcpyToSymbol(g_ct_status, &zero, sizeof(int)) != cudaSuccess) return -1;
  return st;
}

}  // namespace fftgb
