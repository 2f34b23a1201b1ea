// fft3d_fused_tma.cu - pass A of the two-pass 3D FFT (x FFT + NJ-point y
// FFT over rows y = R*j + r of one plane; see fft3d_fused.cu) as a persistent
// kernel fed by the Tensor Memory Accelerator.
//
// The grid is viewed as a 4D tensor [plane][j][r][x] (y = R*j + r), so a
// tile's NJ rows are one box {NX, 1, NJ, 1} at coordinates {0, r, 0, plane}:
// one cp.async.bulk.tensor issued by one thread moves the whole tile (NJ*NX
// points) into shared memory in the [j][x] layout the x FFT reads, and
// completes on an mbarrier with the tile's byte count.  The next tile's copy
// is issued as soon as every thread has read its last-stage inputs of the y
// FFT, so it overlaps the last stage, the stores and the tile switch, as the
// cp.async form (k_xy_pipe) does with eight 16-byte copies per thread.
// The mbarrier waits are bounded (2^24 polls): on a timeout the kernel
// records it in a status word and goes on (results invalid, never a hang).
#include <cuda.h>

#include "fft3d_fused.cuh"
#include "fft3d_fused_cfg.cuh"
#include "tc_core.cuh"

namespace fftgb {

namespace {
constexpr uint32_t XYT_WAIT_LIMIT = 1u << 24;
__device__ int g_xyt_status;
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

int fused_tma_status_and_clear() {
  int st = 0;
  const int zero = 0;
  if (cudaMemcpyFromSymbol(&st, g_xyt_status, sizeof(int)) != cudaSuccess) return -1;
  if (st && cudaMemcpyToSymbol(g_xyt_status, &zero, sizeof(int)) != cudaSuccess) return -1;
  return st;
}

}  // namespace fftgb
