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
#include <string.h>

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

// The tensor maps a launch walks: G = 1, one map over a uniform batch; G =
// FUSED_TMA_GRIDS, one map per grid of a group of same-shape grids at any
// offsets (a ragged batch), tile tl of grid tl / tiles.  Kernel parameters,
// like the single map of the uniform form.
template <int G>
struct XyGrids {
  CUtensorMap in[G];
  long long off[G];  // points from a.out to each grid's output
  long long tiles;   // tiles per grid
};
template <int G>
struct RzGrids {
  CUtensorMap in[G];
  CUtensorMap out[G];
  long long tiles;
};

template <int NX, int NJ, bool INV, int G>
__global__ void __launch_bounds__(XyCfg<NX, NJ>::THREADS, 1024 / XyCfg<NX, NJ>::THREADS)
    k_xy_tma(const FusedArgs a, const __grid_constant__ XyGrids<G> grids, long long ntiles) {
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

  // tile tl -> (grid, plane, residue).  Tile numbers fit 32 bits (the
  // launchers check), so the divisions are 32-bit: a 64-bit division per
  // tile and thread made this issue-bound kernel 20 % slower
  auto locate = [&](long long tl, int &gi, long long &plane, int &r) {
    const unsigned t = (unsigned)tl;
    unsigned lt = t;
    gi = 0;
    if constexpr (G > 1) {
      const unsigned tiles = (unsigned)grids.tiles;
      gi = (int)(t / tiles);
      lt = t - (unsigned)gi * tiles;
    }
    plane = (long long)(lt / (unsigned)R);
    r = (int)(lt - (unsigned)plane * (unsigned)R);
  };
  auto issue = [&](long long tl) {  // one thread
    int gi, r;
    long long pl;
    locate(tl, gi, pl, r);
    const int plane = (int)pl;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(
                     tc::smem_u32(mbar)), "r"(TILE_BYTES) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(tc::smem_u32(tile)),
        "l"(reinterpret_cast<uint64_t>(&grids.in[gi])), "r"(0), "r"(r), "r"(0), "r"(plane),
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
    int gi, r;
    long long plane;
    locate(tl, gi, plane, r);
    float2 *const out = a.out + (G == 1 ? 0 : grids.off[gi]);
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
    float2 *dst = out + (plane * a.ny + (long long)r * NJ) * NX + k;
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
template <int NZ, int R, int X, bool INV, int G>
__global__ void __launch_bounds__(RzTmaCfg<NZ, R, X>::THREADS,
                                  512 / RzTmaCfg<NZ, R, X>::THREADS)
    k_rz_tma(const FusedArgs a, const __grid_constant__ RzGrids<G> grids, long long ntiles) {
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

  // tile tl -> (grid, x block, k1, batch), in 32-bit arithmetic (tile
  // numbers fit 32 bits; the launchers check)
  auto locate = [&](long long tl, int &gi, int &xb, int &k1, long long &bb) {
    const unsigned t = (unsigned)tl;
    unsigned lt = t;
    gi = 0;
    if constexpr (G > 1) {
      const unsigned tiles = (unsigned)grids.tiles;
      gi = (int)(t / tiles);
      lt = t - (unsigned)gi * tiles;
    }
    const unsigned q = lt / (unsigned)xblocks;
    xb = (int)(lt - q * (unsigned)xblocks);
    const unsigned b = q / (unsigned)nj;
    k1 = (int)(q - b * (unsigned)nj);
    bb = (long long)b;
  };
  auto issue = [&](long long tl, int b) {  // one thread
    int gi, xb, k1;
    long long bbl;
    locate(tl, gi, xb, k1, bbl);
    const int bb = (int)bbl;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(
                     tc::smem_u32(mbar + b)), "r"(TILE_BYTES) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4, %5, %6}], [%7];\n" ::"r"(tc::smem_u32(buf + b * TILE)),
        "l"(reinterpret_cast<uint64_t>(&grids.in[gi])), "r"(xb * X), "r"(k1), "r"(0), "r"(0),
        "r"(bb), "r"(tc::smem_u32(mbar + b))
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
    int gi, xb, k1;
    long long bb;
    locate(tl, gi, xb, k1, bb);
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
          "[%0, {%1, %2, %3, %4, %5}], [%6];\n" ::"l"(reinterpret_cast<uint64_t>(&grids.out[gi])),
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
  void (*fn[2])(const FusedArgs, const XyGrids<1>, long long);  // [inverse]
  void (*fng[2])(const FusedArgs, const XyGrids<FUSED_TMA_GRIDS>, long long);
  int threads, smem;
  int grid;
};

#define XYT(NX, NJ)                                                          \
  {NX, NJ, {k_xy_tma<NX, NJ, false, 1>, k_xy_tma<NX, NJ, true, 1>},          \
   {k_xy_tma<NX, NJ, false, FUSED_TMA_GRIDS>, k_xy_tma<NX, NJ, true, FUSED_TMA_GRIDS>}, \
   XyCfg<NX, NJ>::THREADS, XyCfg<NX, NJ>::SMEM + 16, 0}

// NX <= 256: a box dimension holds at most 256 elements
XyTmaEntry kXyTma[] = {
    XYT(256, 64), XYT(256, 32), XYT(128, 128), XYT(128, 64), XYT(64, 64),
    XYT(32, 32), XYT(64, 16),
};
struct RzTmaEntry {
  int nz, r, x;
  void (*fn[2])(const FusedArgs, const RzGrids<1>, long long);
  void (*fng[2])(const FusedArgs, const RzGrids<FUSED_TMA_GRIDS>, long long);
  int threads, smem;
  int grid;
};

#define RZT(NZ, R, X)                                                        \
  {NZ, R, X, {k_rz_tma<NZ, R, X, false, 1>, k_rz_tma<NZ, R, X, true, 1>},    \
   {k_rz_tma<NZ, R, X, false, FUSED_TMA_GRIDS>, k_rz_tma<NZ, R, X, true, FUSED_TMA_GRIDS>}, \
   RzTmaCfg<NZ, R, X>::THREADS, RzTmaCfg<NZ, R, X>::SMEM, 0}

// the pass-B tiles of kRz (fft3d_fused.cu, the fallback for unaligned
// buffers) with R * X == 32
RzTmaEntry kRzTma[] = {RZT(256, 4, 8), RZT(128, 2, 16), RZT(256, 8, 4)};
bool g_tma_ready = false;
EncodeTiledFn g_encode = nullptr;

template <class F>
cudaError_t set_smem_tma(F *fn, int bytes) {
  return cudaFuncSetAttribute((const void *)fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              bytes);
}

// Pass-A map of `planes` planes of one grid shape from `base`: [plane][j][r][x],
// y = R*j + r, strides 8*nx, 8*R*nx, 8*ny*nx bytes
cudaError_t xy_map(CUtensorMap *m, const FusedArgs &a, int nj, const float2 *base,
                   long long planes) {
  const long long R = a.ny / nj;
  const cuuint64_t dims[4] = {(cuuint64_t)a.nx, (cuuint64_t)R, (cuuint64_t)nj,
                              (cuuint64_t)planes};
  const cuuint64_t strides[3] = {(cuuint64_t)a.nx * 8, (cuuint64_t)(R * a.nx * 8),
                                 (cuuint64_t)a.ny * a.nx * 8};
  const cuuint32_t box[4] = {(cuuint32_t)a.nx, 1, (cuuint32_t)nj, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  return g_encode(m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 4, const_cast<float2 *>(base), dims,
                  strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS
             ? cudaSuccess
             : cudaErrorInvalidValue;
}

// Pass-B map of `batch` grids from `base`: [b][z][r][k1][x], y = r*nj + k1,
// strides 8*nx, 8*nj*nx, 8*ny*nx, 8*nz*ny*nx bytes; boxes {X, 1, R, NZ, 1}
cudaError_t rz_map(CUtensorMap *m, const FusedArgs &a, int r, int x, float2 *base,
                   long long batch) {
  const long long nj = a.ny / r;
  const cuuint64_t dims[5] = {(cuuint64_t)a.nx, (cuuint64_t)nj, (cuuint64_t)r,
                              (cuuint64_t)a.nz, (cuuint64_t)batch};
  const cuuint64_t strides[4] = {(cuuint64_t)a.nx * 8, (cuuint64_t)(nj * a.nx * 8),
                                 (cuuint64_t)a.ny * a.nx * 8,
                                 (cuuint64_t)a.nz * a.ny * a.nx * 8};
  const cuuint32_t box[5] = {(cuuint32_t)x, 1, (cuuint32_t)r, (cuuint32_t)a.nz, 1};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  return g_encode(m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 5, base, dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS
             ? cudaSuccess
             : cudaErrorNotSupported;
}
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
    for (int d = 0; d < 2 && e == cudaSuccess; d++) {
      e = set_smem_tma(p.fn[d], p.smem);
      if (e == cudaSuccess) e = set_smem_tma(p.fng[d], p.smem);
    }
    if (e != cudaSuccess) return e;
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, p.fn[0], p.threads, p.smem);
    if (e != cudaSuccess) return e;
    p.grid = (occ > 0 ? occ : 1) * sms;
  }
  for (RzTmaEntry &p : kRzTma) {
    for (int d = 0; d < 2 && e == cudaSuccess; d++) {
      e = set_smem_tma(p.fn[d], p.smem);
      if (e == cudaSuccess) e = set_smem_tma(p.fng[d], p.smem);
    }
    if (e != cudaSuccess) return e;
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
    const long long planes = (long long)a.nz * a.batch;
    const long long ntiles = planes * (a.ny / nj);
    if (ntiles <= 0) return cudaErrorInvalidConfiguration;
    if (ntiles >= (1LL << 31)) return cudaErrorInvalidConfiguration;
    XyGrids<1> g;
    cudaError_t e = xy_map(&g.in[0], a, nj, a.in, planes);
    if (e != cudaSuccess) return e;
    g.off[0] = 0;
    g.tiles = ntiles;
    const int grid = ntiles < p.grid ? (int)ntiles : p.grid;
    return launch_k(p.fn[a.swap_io ? 1 : 0], dim3(grid), dim3(p.threads), p.smem, s, pdl, a,
                    g, ntiles);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_fused_xy_tma_grids(int nj, const FusedArgs &a, const long long *off,
                                      int ngrids, cudaStream_t s, bool pdl) {
  if (!g_tma_ready || !g_encode) return cudaErrorNotSupported;
  if (ngrids < 1 || ngrids > FUSED_TMA_GRIDS) return cudaErrorInvalidValue;
  for (const XyTmaEntry &p : kXyTma) {
    if (p.nx != a.nx || p.nj != nj) continue;
    if (a.ny % nj) return cudaErrorInvalidValue;
    XyGrids<FUSED_TMA_GRIDS> g;
    memset(&g, 0, sizeof(g));
    g.tiles = (long long)a.nz * (a.ny / nj);
    for (int i = 0; i < ngrids; i++) {
      const float2 *base = a.in + off[i];
      if ((uintptr_t)base & 15) return cudaErrorMisalignedAddress;
      const cudaError_t e = xy_map(&g.in[i], a, nj, base, a.nz);
      if (e != cudaSuccess) return e;
      g.off[i] = off[i];
    }
    const long long ntiles = g.tiles * ngrids;
    if (ntiles >= (1LL << 31)) return cudaErrorInvalidConfiguration;
    const int grid = ntiles < p.grid ? (int)ntiles : p.grid;
    return launch_k(p.fng[a.swap_io ? 1 : 0], dim3(grid), dim3(p.threads), p.smem, s, pdl,
                    a, g, ntiles);
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
    const long long ntiles = a.batch * (a.ny / r) * (a.nx / x);
    if (ntiles <= 0) return cudaErrorInvalidConfiguration;
    if (ntiles >= (1LL << 31)) return cudaErrorInvalidConfiguration;
    RzGrids<1> g;
    cudaError_t e = rz_map(&g.in[0], a, r, x, const_cast<float2 *>(a.in), a.batch);
    if (e == cudaSuccess) e = rz_map(&g.out[0], a, r, x, a.out, a.batch);
    if (e != cudaSuccess) return e;
    g.tiles = ntiles;
    const int grid = ntiles < p.grid ? (int)ntiles : p.grid;
    return launch_k(p.fn[a.swap_io ? 1 : 0], dim3(grid), dim3(p.threads), p.smem, s, pdl, a,
                    g, ntiles);
  }
  return cudaErrorNotSupported;
}

cudaError_t launch_fused_rz_tma_grids(int r, int x, const FusedArgs &a, const long long *off,
                                      int ngrids, cudaStream_t s, bool pdl) {
  if (!g_tma_ready || !g_encode) return cudaErrorNotSupported;
  if (ngrids < 1 || ngrids > FUSED_TMA_GRIDS) return cudaErrorInvalidValue;
  for (const RzTmaEntry &p : kRzTma) {
    if (p.nz != a.nz || p.r != r || p.x != x) continue;
    if (a.ny % r || a.nx % x) return cudaErrorInvalidValue;
    RzGrids<FUSED_TMA_GRIDS> g;
    memset(&g, 0, sizeof(g));
    g.tiles = (long long)(a.ny / r) * (a.nx / x);
    for (int i = 0; i < ngrids; i++) {
      float2 *bi = const_cast<float2 *>(a.in) + off[i];
      float2 *bo = a.out + off[i];
      if (((uintptr_t)bi | (uintptr_t)bo) & 15) return cudaErrorMisalignedAddress;
      cudaError_t e = rz_map(&g.in[i], a, r, x, bi, 1);
      if (e == cudaSuccess) e = rz_map(&g.out[i], a, r, x, bo, 1);
      if (e != cudaSuccess) return e;
    }
    const long long ntiles = g.tiles * ngrids;
    if (ntiles >= (1LL << 31)) return cudaErrorInvalidConfiguration;
    const int grid = ntiles < p.grid ? (int)ntiles : p.grid;
    return launch_k(p.fng[a.swap_io ? 1 : 0], dim3(grid), dim3(p.threads), p.smem, s, pdl,
                    a, g, ntiles);
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
