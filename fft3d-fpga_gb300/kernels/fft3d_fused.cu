// fft3d_fused.cu - two-pass 3D FFT: every point crosses HBM twice (read +
// write per pass), the minimum for grids larger than on-chip memory.
//
// The reference runs x, y and z through three engines with an on-chip xy
// transpose and a DDR yz transpose in between (kernels/fft3d/fft3d_ddr.cl:
// 69-416).  Here the y axis is split between the two passes (four-step
// decomposition, y = R*j + r, k = k1 + (NY/R)*k2):
//
//   pass A, k_xy<NX, NJ>: one CTA per (plane, residue r) loads the NJ = NY/R
//     rows y = R*j + r, runs the x-FFT of every row, then the length-NJ FFT
//     over j of every column, multiplies by W_NY^(r*k1) and stores row
//     r*NJ + k1 of the plane (contiguous rows, coalesced).
//   pass B, k_rz<NZ, R, X>: one CTA per (batch, k1, X-column block) loads the
//     R rows {r*NJ + k1} of every plane, combines them with a radix-R DFT
//     into rows k1 + NJ*k2, then runs the z-FFT of each (row, column) and
//     stores in natural order.  It reads and writes the same rows, so it runs
//     in place on the output buffer.
//
// Both tiles live in shared memory; HBM is touched only by the first loads
// and the last stores of each pass.
#include "fft_core.cuh"
#include "filter.cuh"
#include "fft3d_fused.cuh"
#include "fft3d_fused_cfg.cuh"

namespace fftgb {

// Pass-A tile (plane, r): rows y = R*j + r of one plane; EP points per thread.
template <int NX, int NJ, bool INV, int EP = 16>
__device__ __forceinline__ void xy_tile(const FusedArgs &a, long long bid, float2 *tile) {
  using K = XyCfg<NX, NJ, EP>;
  using CX = typename K::CX;
  using CJ = typename K::CJ;
  constexpr int E = K::E;
  const int tid = threadIdx.x;
  const int R = a.ny / NJ;
  // bid is a block index (< 2^31): 32-bit division
  const long long plane = (unsigned)bid / (unsigned)R;
  const int r = (int)((unsigned)bid - (unsigned)plane * (unsigned)R);

  // ---- x-FFT of row j (global row y = R*j + r)
  {
    const int j = tid / CX::T;
    const int t = tid - j * CX::T;
    const float2 *src = a.in + (plane * a.ny + (long long)R * j + r) * NX;
    float2 v[E];
#pragma unroll
    for (int q = 0; q < E; q++) {
      const float2 x = src[in_index<CX>(t, q)];
      v[q] = INV ? cswap(x) : x;
    }
    float2 *row = tile + j * NX;
    stockham_row<CX, NJ>(v, t, [row](int i) -> float2 & { return row[swz(i)]; },
                         a.tw_x, j);
    row_sync<CX, NJ>(j);
#pragma unroll
    for (int q = 0; q < E; q++) tile[j * NX + out_index<CX>(t, q)] = v[q];
  }
  __syncthreads();

  // ---- y-FFT over j of column k, twiddle, store row r*NJ + k1
  if constexpr (NJ < 16) {
    // short y transforms (2D tiles of fewer than 16 rows): every thread
    // takes 16 / NJ whole columns and transforms them in registers
    constexpr int THREADS = K::THREADS;
    static_assert(EP == 16, "short y transforms with 16 points per thread");
    constexpr int CPT = 16 / NJ;
    static_assert(THREADS * CPT == NX, "columns per thread");
#pragma unroll
    for (int c = 0; c < CPT; c++) {
      const int k = tid + c * THREADS;
      float2 v[NJ];
#pragma unroll
      for (int j = 0; j < NJ; j++) v[j] = tile[j * NX + k];
      dft<NJ>(v);
      float2 *dst = a.out + (plane * a.ny + (long long)r * NJ) * NX + k;
#pragma unroll
      for (int k1 = 0; k1 < NJ; k1++) {
        float2 x = v[k1];
        if (R > 1 && !a.twb) x = cmul(x, __ldg(&a.tw_y[r * k1]));
        if (a.scale != 1.0f) x = cscale(x, a.scale);
        dst[(long long)k1 * NX] = INV ? cswap(x) : x;
      }
    }
  } else {
    const int k = tid % NX;
    const int t = tid / NX;
    float2 v[E];
#pragma unroll
    for (int q = 0; q < E; q++) v[q] = tile[in_index<CJ>(t, q) * NX + k];
    __syncthreads();
    stockham<CJ>(v, t, [k](int i) -> float2 & {
      extern __shared__ float2 tile_[];
      return tile_[i * NX + k];
    }, a.tw_j);
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
}

template <int NX, int NJ, bool INV, int EP = 16>
__global__ void __launch_bounds__(XyCfg<NX, NJ, EP>::THREADS,
                                  XyCfg<NX, NJ, EP>::THREADS == 512 ? 2 : 1)
    k_xy(const FusedArgs a) {
  extern __shared__ float2 tile[];
  pdl_enter();
  xy_tile<NX, NJ, INV, EP>(a, blockIdx.x, tile);
}

// Pass-B tile (batch, k1, x block); EP points per thread.
template <int NZ, int R, int X, bool INV, int EP = 16>
__device__ __forceinline__ void rz_tile(const FusedArgs &a, long long bid, float2 *tile) {
  using K = RzCfg<NZ, R, X, EP>;
  using CZ = typename K::CZ;
  constexpr int E = K::E;
  constexpr int THREADS = K::THREADS;
  const int tid = threadIdx.x;
  const int nj = a.ny / R;
  const int xblocks = a.nx / X;
  // bid is a block index (< 2^31): 32-bit divisions
  const unsigned q = (unsigned)bid / (unsigned)xblocks;
  const int xb = (int)((unsigned)bid - q * (unsigned)xblocks);
  const unsigned bq = q / (unsigned)nj;
  const int k1 = (int)(q - bq * (unsigned)nj);
  const long long b = bq;
  const long long plane_pts = (long long)a.ny * a.nx;
  const float2 *src = a.in + b * NZ * plane_pts + (long long)k1 * a.nx + xb * X;
  float2 *dst = a.out + b * NZ * plane_pts + (long long)k1 * a.nx + xb * X;

  const int x = tid % X;
  float2 v[E];
  if constexpr (R > 1) {
    // ---- radix-R over the residue rows r*nj + k1 -> rows k1 + nj*k2
    constexpr int ITEMS = E / R;
    constexpr int ZSTEP = THREADS / X;
    const int z0 = tid / X;
    float2 wr[R];  // W_ny^(rr*k1) when pass A left it to this pass
#pragma unroll
    for (int rr = 1; rr < R; rr++)
      wr[rr] = a.twb ? __ldg(&a.tw_y[rr * k1]) : make_float2(1.f, 0.f);
#pragma unroll
    for (int m = 0; m < ITEMS; m++) {
      const int z = z0 + m * ZSTEP;
      float2 u[R];
#pragma unroll
      for (int rr = 0; rr < R; rr++) {
        const float2 w = src[z * plane_pts + (long long)rr * nj * a.nx + x];
        u[rr] = INV ? cswap(w) : w;
        if (rr > 0 && a.twb) u[rr] = cmul(u[rr], wr[rr]);
      }
      dft<R>(u);
#pragma unroll
      for (int k2 = 0; k2 < R; k2++) tile[k2 * K::KS + z * X + x] = u[k2];
    }
    __syncthreads();
    const int k2 = (tid / X) % R;
    const int t = tid / (X * R);
#pragma unroll
    for (int q = 0; q < E; q++) v[q] = tile[k2 * K::KS + in_index<CZ>(t, q) * X + x];
    __syncthreads();
    stockham<CZ>(v, t, [k2, x](int i) -> float2 & {
      extern __shared__ float2 tile_[];
      return tile_[k2 * K::KS + i * X + x];
    }, a.tw_z);
    float2 *d = dst + (long long)k2 * nj * a.nx;
#pragma unroll
    for (int q = 0; q < E; q++) {
      float2 w = v[q];
      if (a.scale != 1.0f) w = cscale(w, a.scale);
      if (a.filter)
        w = cscale(w, filter_g(a.filter, xb * X + x, k1 + nj * k2, out_index<CZ>(t, q), a.nx,
                               a.ny, NZ));
      d[out_index<CZ>(t, q) * plane_pts + x] = INV ? cswap(w) : w;
    }
  } else {
    // ---- plain z-FFT of X columns of row k1
    const int t = tid / X;
#pragma unroll
    for (int q = 0; q < E; q++) {
      const float2 w = src[in_index<CZ>(t, q) * plane_pts + x];
      v[q] = INV ? cswap(w) : w;
    }
    stockham<CZ>(v, t, [x](int i) -> float2 & {
      extern __shared__ float2 tile_[];
      return tile_[i * X + x];
    }, a.tw_z);
#pragma unroll
    for (int q = 0; q < E; q++) {
      float2 w = v[q];
      if (a.scale != 1.0f) w = cscale(w, a.scale);
      if (a.filter)
        w = cscale(w, filter_g(a.filter, xb * X + x, k1, out_index<CZ>(t, q), a.nx, a.ny, NZ));
      dst[out_index<CZ>(t, q) * plane_pts + x] = INV ? cswap(w) : w;
    }
  }
}

template <int NZ, int R, int X, bool INV, int EP = 16>
__global__ void __launch_bounds__(RzCfg<NZ, R, X, EP>::THREADS,
                                  RzCfg<NZ, R, X, EP>::THREADS == 512 ? 2 : 1)
    k_rz(const FusedArgs a) {
  extern __shared__ float2 tile[];
  pdl_enter();
  rz_tile<NZ, R, X, INV, EP>(a, blockIdx.x, tile);
}

// ------------------------------------------------------------ dispatch
namespace {
template <class F>
cudaError_t set_smem(F *fn, int bytes) {
  return cudaFuncSetAttribute((const void *)fn,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

struct XyEntry {
  int nx, nj, e;
  void (*fn[2])(const FusedArgs);  // [inverse]
  int threads, smem;
};
struct RzEntry {
  int nz, r, x, e;
  void (*fn[2])(const FusedArgs);
  int threads, smem;
};

#define XYE(NX, NJ, E)                                                         \
  {NX, NJ, E, {k_xy<NX, NJ, false, E>, k_xy<NX, NJ, true, E>}, XyCfg<NX, NJ, E>::THREADS, \
   XyCfg<NX, NJ, E>::SMEM}
#define XY(NX, NJ) XYE(NX, NJ, 16)
#define RZE(NZ, R, X, E)                                                       \
  {NZ, R, X, E, {k_rz<NZ, R, X, false, E>, k_rz<NZ, R, X, true, E>},            \
   RzCfg<NZ, R, X, E>::THREADS, RzCfg<NZ, R, X, E>::SMEM}
#define RZ(NZ, R, X) RZE(NZ, R, X, 16)

XyEntry kXy[] = {
    XY(256, 64), XY(128, 128), XY(64, 64), XY(256, 32), XY(128, 64),
    XY(1024, 16), XY(512, 32), XY(32, 32), XY(64, 16),
    XY(1024, 8), XY(512, 16), XY(2048, 8), XY(2048, 4),
    // 8 points per thread: 64^3 (at 128^3 the 16-point tiles lead: 4 x 128^3
    // pass A 0.049 against 0.039 ms)
    XYE(64, 64, 8),
};
RzEntry kRz[] = {
    RZ(256, 4, 16), RZ(256, 8, 8), RZ(128, 1, 64), RZ(64, 1, 64),
    RZ(256, 2, 32), RZ(128, 2, 32), RZ(32, 1, 32),
    RZ(256, 8, 4), RZ(256, 4, 8), RZ(128, 1, 32), RZ(64, 1, 32),
    RZ(128, 2, 16),
    RZE(64, 1, 32, 8),
};
bool g_fused_ready = false;
}  // namespace

cudaError_t fused_kernels_init() {
  if (g_fused_ready) return cudaSuccess;
  cudaError_t r = cudaSuccess;
  for (XyEntry &e : kXy)
    for (int d = 0; d < 2 && r == cudaSuccess; d++) r = set_smem(e.fn[d], e.smem);
  for (RzEntry &e : kRz)
    for (int d = 0; d < 2 && r == cudaSuccess; d++) r = set_smem(e.fn[d], e.smem);
  if (r != cudaSuccess) return r;
  g_fused_ready = true;
  return cudaSuccess;
}

bool fused_xy_available(int nx, int nj, int ept) {
  for (const XyEntry &e : kXy)
    if (e.nx == nx && e.nj == nj && e.e == ept) return true;
  return false;
}

bool fused_rz_available(int nz, int r, int x, int ept) {
  for (const RzEntry &e : kRz)
    if (e.nz == nz && e.r == r && e.x == x && e.e == ept) return true;
  return false;
}

cudaError_t launch_fused_xy(int nj, const FusedArgs &a, cudaStream_t s, bool pdl, int ept) {
  if (!g_fused_ready) return cudaErrorInvalidValue;
  for (const XyEntry &e : kXy) {
    if (e.nx == a.nx && e.nj == nj && e.e == ept) {
      if (a.ny % nj) return cudaErrorInvalidValue;
      const long long grid = (long long)a.nz * a.batch * (a.ny / nj);
      if (grid <= 0 || grid > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
      return launch_k(e.fn[a.swap_io ? 1 : 0], dim3((unsigned)grid), dim3(e.threads),
                      e.smem, s, pdl, a);
    }
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_fused_rz(int r, int x, const FusedArgs &a, cudaStream_t s, bool pdl,
                            int ept) {
  if (!g_fused_ready) return cudaErrorInvalidValue;
  for (const RzEntry &e : kRz) {
    if (e.nz == a.nz && e.r == r && e.x == x && e.e == ept) {
      if (a.ny % r || a.nx % x) return cudaErrorInvalidValue;
      const long long grid = (long long)a.batch * (a.ny / r) * (a.nx / x);
      if (grid <= 0 || grid > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
      return launch_k(e.fn[a.swap_io ? 1 : 0], dim3((unsigned)grid), dim3(e.threads),
                      e.smem, s, pdl, a);
    }
  }
  return cudaErrorInvalidValue;
}

}  // namespace fftgb
