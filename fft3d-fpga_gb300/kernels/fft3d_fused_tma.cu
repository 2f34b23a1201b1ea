// fft3d_fused_tma.cu - passes A and B of the two-pass 3D FFT (pass A: x FFT
// + NJ-point y FFT over rows y = R*j + r of one plane; pass B: radix-R over
// the residue rows + z FFT; see fft3d_fused.cu) as persistent kernels fed by
// the Tensor Memory Accelerator.  Pass A first, pass B below.
//
// The grid is viewed as a 4D tensor [plane][j][r][x] (y = R*j + r), so a
// tile's NJ rows are one box {NX, 1, NJ, 1} at coordinates {0, r, 0, plane}:
// one cp.async.bulk.tensor issued by one thread moves the whole tile (NJ*NX
// points) into shared memory in the [j][x] layout the x FFT reads, and
// completes on an mbarrier with the tile's byte count.  The next tile's copy
// is issued as soon as every thread has read its last-stage inputs of the y
// FFT, so it overlaps the last stage, the stores and the tile switch (a
// cp.async form with eight 16-byte copies per thread measured slower).
// The mbarrier waits are bounded (2^24 polls): on a timeout the kernel
// records it in a status word and goes on (results invalid, never a hang).
#include <cuda.h>

#include "filter.cuh"
#include "fft3d_fused.cuh"
#include "fft3d_fused_cfg.cuh"
#include "tc_core.cuh"

namespace fftgb {

namespace {
constexpr uint32_t XYT_WAIT_LIMIT = 1u << 24;
__device__ int g_xyt_status;
__global__ void k_fused_tma_expire(uint32_t polls) { tc::expire_wait(&g_xyt_status, polls); }
}  // namespace

template <int NX, int NJ, bool INV>
__global__ void __launch_bounds__(XyCfg<NX, NJ>::THREADS, 1024 / XyCfg<NX, NJ>::THREADS)
    k_xy_tma(const FusedArgs a, const __grid_constant__ CUtensorMap tmap, long long ntiles) {
  using K = XyCfg<NX, NJ>;
  using CX = typename K::CX;
  using CJ = typename K::CJ;
  constexpr int E = K::E;
  constexpr uint32_t TILE_BYTES = (uint32_t)(NJ * NX * sizeof(float2));
  extern __shared__ __align__(128) float2 tile[];
  uint64_t *mbar = reinterpret_cast<uint64_t *>(tile + NJ * NX);
  pdl_enter();
  const int tid = threadIdx.x;
  const int R = a.ny / NJ;

  auto issue = [&](long long tl) {  // one thread
    const int plane = (int)(tl / R);
    const int r = (int)(tl - (long long)plane * R);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(
                     tc::smem_u32(mbar)), "r"(TILE_BYTES) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(tc::smem_u32(tile)),
        "l"(reinterpret_cast<uint64_t>(&tmap)), "r"(0), "r"(r), "r"(0), "r"(plane),
        "r"(tc::smem_u32(mbar))
        : "memory");
  };

  if (tid == 0) {
    tc::mbar_init(mbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    if (blockIdx.x < ntiles) issue(blockIdx.x);
  }
  __syncthreads();  // the mbarrier is initialised before anyone waits on it

  bool ok = true;
  uint32_t phase = 0;
  for (long long tl = blockIdx.x; tl < ntiles; tl += gridDim.x) {
    const long long plane = tl / R;
    const int r = (int)(tl - plane * R);
    ok = tc::mbar_wait_bounded(mbar, phase, XYT_WAIT_LIMIT) && ok;
    phase ^= 1u;

    // ---- x-FFT of row j
    {
      const int j = tid / CX::T;
      const int t = tid - j * CX::T;
      float2 v[E];
#pragma unroll
      for (int q = 0; q < E; q++) {
        const float2 x = tile[j * NX + in_index<CX>(t, q)];
        v[q] = INV ? cswap(x) : x;
      }
      row_sync<CX, NJ>(j);  // this row's raw reads done before its exchange
      float2 *row = tile + j * NX;
      stockham_row<CX, NJ>(v, t, [row](int i) -> float2 & { return row[swz(i)]; }, a.tw_x, j);
      row_sync<CX, NJ>(j);
#pragma unroll
      for (int q = 0; q < E; q++) tile[j * NX + out_index<CX>(t, q)] = v[q];
    }
    __syncthreads();

    // ---- y-FFT over j of column k, twiddle, store row r*NJ + k1
    const int k = tid % NX;
    const int t = tid / NX;
    float2 v[E];
#pragma unroll
    for (int q = 0; q < E; q++) v[q] = tile[in_index<CJ>(t, q) * NX + k];
    __syncthreads();
    const long long next = tl + gridDim.x;
    auto hook = [&]() {
      // every thread has read its last-stage inputs: order these generic
      // accesses before the tensor copy that overwrites the tile
      tc::fence_proxy_async();
      __syncthreads();
      if (tid == 0 && next < ntiles) issue(next);
    };
    stockham_h<CJ>(v, t, [k](int i) -> float2 & {
      extern __shared__ __align__(128) float2 tile_[];
      return tile_[i * NX + k];
    }, a.tw_j, hook);
    float2 *dst = a.out + (plane * a.ny + (long long)r * NJ) * NX + k;
#pragma unroll
    for (int q = 0; q < E; q++) {
      const int k1 = out_index<CJ>(t, q);
      float2 x = v[q];
      if (R > 1 && !a.twb) x = cmul(x, __ldg(&a.tw_y[r * k1]));
      if (a.scale != 1.0f) x = cscale(x, a.scale);
      dst[(long long)k1 * NX] = INV ? cswap(x) : x;
    }
  }
  if (!ok) atomicExch(&g_xyt_status, 1);
}

// ---------------------------------------------------------------- pass B
// Pass B (radix-R over the residue rows y = r*nj + k1 of one x block, then
// the NZ-point z FFT of every resulting row; see rz_tile in fft3d_fused.cu)
// as a persistent kernel with three tile buffers fed and drained by TMA.
// The pass-B input is viewed as a 5D tensor [b][z][r][k1][x]; a tile (b, k1,
// x block) is one box {X, 1, R, NZ, 1}, which lands as [z][r][x]: with
// R*X = 32 a warp's
// lanes are the (x, r) pairs of one z, so every shared access of a warp is
// 32 consecutive points (no bank conflicts).  The radix-R step runs across
// lanes: lane (x, r) holds input row r of its 16 z points, R/2-apart lanes
// exchange values by shuffles in the decimation-in-frequency order, and lane
// r ends with output row bitrev(r); the z FFT then uses the lane's own
// column of the buffer for its exchanges.  A tile's input and output cover
// the same rows, so tiles are disjoint and the pass may run in place.
template <int NZ, int R, int X>
struct RzTmaCfg {
  using CZ = Stock<NZ, 16>;
  static constexpr int THREADS = 32 * CZ::T;
  static constexpr int TILE = NZ * R * X;  // points
  static constexpr int NBUF = 3;
  static constexpr int SMEM = NBUF * TILE * (int)sizeof(float2) + 32;
  static_assert(R * X == 32, "one warp spans the (x, r) pairs of one z");
  static_assert(R == 2 || R == 4 || R == 8, "lane radix 2, 4 or 8");
  static_assert(THREADS <= 512, "z FFT of at most 256 points");
};

// The outputs go back into the tile's buffer and out by one TMA tensor store
// per tile; with three buffers a buffer is refilled (tile i + 2 into the
// buffer of tile i - 1) only once its store has read it.  Against per-thread
// stores of the 64-byte output runs: 256^3 x 8 pass B 0.378 against
// 0.403 ms, 128^3 x 4 0.026 against 0.028.
template <int NZ, int R, int X, bool INV>
__global__ void __launch_bounds__(RzTmaCfg<NZ, R, X>::THREADS,
                                  512 / RzTmaCfg<NZ, R, X>::THREADS)
    k_rz_tma(const FusedArgs a, const __grid_constant__ CUtensorMap tmap,
             const __grid_constant__ CUtensorMap tmap_out, long long ntiles) {
  using K = RzTmaCfg<NZ, R, X>;
  using CZ = typename K::CZ;
  constexpr int E = 16, TILE = K::TILE, NBUF = K::NBUF;
  constexpr uint32_t TILE_BYTES = (uint32_t)(TILE * sizeof(float2));
  extern __shared__ __align__(128) float2 buf[];
  uint64_t *mbar = reinterpret_cast<uint64_t *>(buf + NBUF * TILE);
  pdl_enter();
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int t = tid >> 5;
  const int x = lane % X;
  // the lane groups of X lanes hold the rows r so that a half-warp's rows
  // have their X-point runs in disjoint banks both in the input order r and
  // in the output order bitrev(r): R = 4 groups 0..3 hold r = 0, 3, 1, 2
  // (half-warps {0, 3}, {1, 2}); R = 8 groups 0..7 hold r = 0, 2, 5, 7, 4,
  // 6, 1, 3 (r = g1 + 2 g0 + 4 (g1 xor g2) for group g = 4 g2 + 2 g1 + g0)
  const int g = lane / X;
  const int r = (R == 8)   ? (((g >> 1) & 1) | ((g & 1) << 1) | ((((g >> 1) ^ (g >> 2)) & 1) << 2))
                : (R == 4) ? (((g & 1) << 1) | ((g ^ (g >> 1)) & 1))
                           : g;
  const int nj = a.ny / R;
  const int xblocks = a.nx / X;

  auto issue = [&](long long tl, int b) {  // one thread
    const int xb = (int)(tl % xblocks);
    const int k1 = (int)((tl / xblocks) % nj);
    const int bb = (int)(tl / ((long long)xblocks * nj));
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(
                     tc::smem_u32(mbar + b)), "r"(TILE_BYTES) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4, %5, %6}], [%7];\n" ::"r"(tc::smem_u32(buf + b * TILE)),
        "l"(reinterpret_cast<uint64_t>(&tmap)), "r"(xb * X), "r"(k1), "r"(0), "r"(0), "r"(bb),
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
    const int xb = (int)(tl % xblocks);
    const int k1 = (int)((tl / xblocks) % nj);
    const long long bb = tl / ((long long)xblocks * nj);
    // W_ny^(r*k1) when pass A left the y twiddle to this pass
    const float2 wr = (a.twb && r > 0) ? __ldg(&a.tw_y[r * k1]) : make_float2(1.f, 0.f);
    ok = tc::mbar_wait_bounded(mbar + b, (phases >> b) & 1u, XYT_WAIT_LIMIT) && ok;
    phases ^= 1u << b;

    float2 v[E];
#pragma unroll
    for (int q = 0; q < E; q++) {
      const float2 w = tile[in_index<CZ>(t, q) * 32 + r * X + x];
      v[q] = cmul(INV ? cswap(w) : w, wr);
    }
    __syncthreads();  // every stage-0 input read before the in-place exchange
    // radix-R over r across the lanes (decimation in frequency): the lane
    // with bit h of r clear keeps a + b, the other (a - b) * W_2h^(r mod h),
    // both as s*own + partner with s = -1 on the second (one FMA a value).
    // The partner (r xor h) is 3X lanes away for h = 2, 2X for h = 1 when
    // R = 4; 4X for h = 4, X for h = 2, 6X for h = 1 when R = 8
#pragma unroll
    for (int h = R / 2; h >= 1; h >>= 1) {
      const float s = (r & h) ? -1.f : 1.f;
      const bool rot = h == 2 && (r & 3) == 3;  // W_4^1 = -i
      const int pm = (R == 8)   ? (h == 4 ? 4 * X : h == 2 ? X : 6 * X)
                     : (R == 4) ? (h == 2 ? 3 * X : 2 * X)
                                : X;
      // h = 4: W_8^(r mod 4) on the lanes with bit 2 of r set
      constexpr float C8 = 0.70710678118654752f;
      const float2 w8 = (h != 4 || !(r & 4)) ? make_float2(1.f, 0.f)
                        : (r & 3) == 0       ? make_float2(1.f, 0.f)
                        : (r & 3) == 1       ? make_float2(C8, -C8)
                        : (r & 3) == 2       ? make_float2(0.f, -1.f)
                                             : make_float2(-C8, -C8);
#pragma unroll
      for (int q = 0; q < E; q++) {
        const float px = __shfl_xor_sync(0xffffffffu, v[q].x, pm);
        const float py = __shfl_xor_sync(0xffffffffu, v[q].y, pm);
        float2 o = make_float2(fmaf(s, v[q].x, px), fmaf(s, v[q].y, py));
        if (h == 4) o = cmul(o, w8);
        v[q] = rot ? make_float2(o.y, -o.x) : o;
      }
    }
    const int k2 = (R == 8)   ? (((r & 1) << 2) | (r & 2) | (r >> 2))
                   : (R == 4) ? (((r & 1) << 1) | (r >> 1))
                              : r;  // bitrev(r)
    stockham<CZ>(v, t, [tile, lane](int m) -> float2 & { return tile[m * 32 + lane]; },
                 a.tw_z);
    __syncthreads();  // every last-stage input read before the outputs land
#pragma unroll
    for (int q = 0; q < E; q++) {
      float2 w = v[q];
      if (a.scale != 1.0f) w = cscale(w, a.scale);
      if (a.filter)
        w = cscale(w, filter_g(a.filter, xb * X + x, k1 + nj * k2, out_index<CZ>(t, q), a.nx,
                               a.ny, a.nz));
      tile[out_index<CZ>(t, q) * 32 + k2 * X + x] = INV ? cswap(w) : w;
    }
    // order the generic writes before the tensor store that reads them
    tc::fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      asm volatile(
          "cp.async.bulk.tensor.5d.global.shared::cta.bulk_group "
          "[%0, {%1, %2, %3, %4, %5}], [%6];\n" ::"l"(reinterpret_cast<uint64_t>(&tmap_out)),
          "r"(xb * X), "r"(k1), "r"(0), "r"(0), "r"((int)bb), "r"(tc::smem_u32(tile))
          : "memory");
      asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
      // the previous tile's store has read its buffer, which takes the tile
      // after next
      asm volatile("cp.async.bulk.wait_group.read 1;\n" ::: "memory");
      const long long after = tl + 2 * (long long)gridDim.x;
      if (after < ntiles) issue(after, b == 0 ? NBUF - 1 : b - 1);
    }
    b = (b + 1 == NBUF) ? 0 : b + 1;
  }
  // the last stores complete before the CTA (and its shared memory) ends
  if (tid == 0) asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
  if (!ok) atomicExch(&g_xyt_status, 1);
}

namespace {
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion,
                                  CUtensorMapFloatOOBfill);

struct XyTmaEntry {
  int nx, nj;
  void (*fn[2])(const FusedArgs, const CUtensorMap, long long);
  int threads, smem;
  int grid;
};

#define XYT(NX, NJ)                                                          \
  {NX, NJ, {k_xy_tma<NX, NJ, false>, k_xy_tma<NX, NJ, true>},                \
   XyCfg<NX, NJ>::THREADS, XyCfg<NX, NJ>::SMEM + 16, 0}

// NX <= 256: a box dimension holds at most 256 elements
XyTmaEntry kXyTma[] = {
    XYT(256, 64), XYT(256, 32), XYT(128, 128), XYT(128, 64), XYT(64, 64),
    XYT(32, 32), XYT(64, 16),
};
struct RzTmaEntry {
  int nz, r, x;
  void (*fn[2])(const FusedArgs, const CUtensorMap, const CUtensorMap, long long);
  int threads, smem;
  int grid;
};

#define RZT(NZ, R, X)                                                        \
  {NZ, R, X, {k_rz_tma<NZ, R, X, false>, k_rz_tma<NZ, R, X, true>},          \
   RzTmaCfg<NZ, R, X>::THREADS, RzTmaCfg<NZ, R, X>::SMEM, 0}

// the pass-B tiles of kRz (fft3d_fused.cu, the fallback for unaligned
// buffers) with R * X == 32
RzTmaEntry kRzTma[] = {RZT(256, 4, 8), RZT(128, 2, 16), RZT(256, 8, 4)};
bool g_tma_ready = false;
EncodeTiledFn g_encode = nullptr;
}  // namespace

cudaError_t fused_tma_init() {
  if (g_tma_ready) return cudaSuccess;
  void *fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                       &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess)
    fn = nullptr;
  cudaGetLastError();
  g_encode = reinterpret_cast<EncodeTiledFn>(fn);
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  for (XyTmaEntry &p : kXyTma) {
    for (int d = 0; d < 2; d++) {
      e = cudaFuncSetAttribute((const void *)p.fn[d],
                               cudaFuncAttributeMaxDynamicSharedMemorySize, p.smem);
      if (e != cudaSuccess) return e;
    }
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, p.fn[0], p.threads, p.smem);
    if (e != cudaSuccess) return e;
    p.grid = (occ > 0 ? occ : 1) * sms;
  }
  for (RzTmaEntry &p : kRzTma) {
    for (int d = 0; d < 2; d++) {
      e = cudaFuncSetAttribute((const void *)p.fn[d],
                               cudaFuncAttributeMaxDynamicSharedMemorySize, p.smem);
      if (e != cudaSuccess) return e;
    }
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, p.fn[0], p.threads, p.smem);
    if (e != cudaSuccess) return e;
    p.grid = (occ > 0 ? occ : 1) * sms;
  }
  g_tma_ready = true;
  return cudaSuccess;
}

bool fused_xy_tma_available(int nx, int nj) {
  if (!g_encode) return false;
  for (const XyTmaEntry &p : kXyTma)
    if (p.nx == nx && p.nj == nj) return true;
  return false;
}

cudaError_t launch_fused_xy_tma(int nj, const FusedArgs &a, cudaStream_t s, bool pdl) {
  if (!g_tma_ready || !g_encode) return cudaErrorNotSupported;
  // the tensor's base must be 16-byte aligned (the output is written with
  // plain stores)
  if ((uintptr_t)a.in & 15) return cudaErrorMisalignedAddress;
  for (const XyTmaEntry &p : kXyTma) {
    if (p.nx != a.nx || p.nj != nj) continue;
    if (a.ny % nj) return cudaErrorInvalidValue;
    const long long R = a.ny / nj;
    const long long planes = (long long)a.nz * a.batch;
    const long long ntiles = planes * R;
    if (ntiles <= 0) return cudaErrorInvalidConfiguration;
    // [plane][j][r][x], y = R*j + r: strides 8*nx, 8*R*nx, 8*ny*nx bytes
    const cuuint64_t dims[4] = {(cuuint64_t)a.nx, (cuuint64_t)R, (cuuint64_t)nj,
                                (cuuint64_t)planes};
    const cuuint64_t strides[3] = {(cuuint64_t)a.nx * 8, (cuuint64_t)(R * a.nx * 8),
                                   (cuuint64_t)a.ny * a.nx * 8};
    const cuuint32_t box[4] = {(cuuint32_t)a.nx, 1, (cuuint32_t)nj, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    CUtensorMap m;
    if (g_encode(&m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 4, const_cast<float2 *>(a.in), dims,
                 strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return cudaErrorInvalidValue;
    const int grid = ntiles < p.grid ? (int)ntiles : p.grid;
    return launch_k(p.fn[a.swap_io ? 1 : 0], dim3(grid), dim3(p.threads), p.smem, s, pdl, a,
                    m, ntiles);
  }
  return cudaErrorInvalidValue;
}

bool fused_rz_tma_available(int nz, int r, int x) {
  if (!g_encode) return false;
  for (const RzTmaEntry &p : kRzTma)
    if (p.nz == nz && p.r == r && p.x == x) return true;
  return false;
}

cudaError_t launch_fused_rz_tma(int r, int x, const FusedArgs &a, cudaStream_t s, bool pdl) {
  if (!g_tma_ready || !g_encode) return cudaErrorNotSupported;
  // both tensor maps need 16-byte aligned bases
  if (((uintptr_t)a.in | (uintptr_t)a.out) & 15) return cudaErrorMisalignedAddress;
  for (const RzTmaEntry &p : kRzTma) {
    if (p.nz != a.nz || p.r != r || p.x != x) continue;
    if (a.ny % r || a.nx % x) return cudaErrorInvalidValue;
    const long long nj = a.ny / r;
    const long long ntiles = a.batch * nj * (a.nx / x);
    if (ntiles <= 0) return cudaErrorInvalidConfiguration;
    // [b][z][r][k1][x], y = r*nj + k1: strides 8*nx, 8*nj*nx, 8*ny*nx,
    // 8*nz*ny*nx bytes
    const cuuint64_t dims[5] = {(cuuint64_t)a.nx, (cuuint64_t)nj, (cuuint64_t)r,
                                (cuuint64_t)a.nz, (cuuint64_t)a.batch};
    const cuuint64_t strides[4] = {(cuuint64_t)a.nx * 8, (cuuint64_t)(nj * a.nx * 8),
                                   (cuuint64_t)a.ny * a.nx * 8,
                                   (cuuint64_t)a.nz * a.ny * a.nx * 8};
    const cuuint32_t box[5] = {(cuuint32_t)x, 1, (cuuint32_t)r, (cuuint32_t)a.nz, 1};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    CUtensorMap m, mo;
    if (g_encode(&m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 5, const_cast<float2 *>(a.in), dims,
                 strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return cudaErrorNotSupported;
    if (g_encode(&mo, CU_TENSOR_MAP_DATA_TYPE_UINT64, 5, a.out, dims, strides, box, estr,
                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return cudaErrorNotSupported;
    const int grid = ntiles < p.grid ? (int)ntiles : p.grid;
    return launch_k(p.fn[a.swap_io ? 1 : 0], dim3(grid), dim3(p.threads), p.smem, s, pdl, a,
                    m, mo, ntiles);
  }
  return cudaErrorNotSupported;
}

cudaError_t fused_tma_expire_wait(unsigned polls) {
  k_fused_tma_expire<<<1, 32>>>(polls);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? cudaDeviceSynchronize() : e;
}

int fused_tma_status_and_clear() {
  int st = 0;
  const int zero = 0;
  if (cudaMemcpyFromSymbol(&st, g_xyt_status, sizeof(int)) != cudaSuccess) return -1;
  if (st && cudaMemcpyToSymbol(g_xyt_status, &zero, sizeof(int)) != cudaSuccess) return -1;
  return st;
}

}  // namespace fftgb
