// fft3d_fused_pipe.cu - persistent, software-pipelined forms of passes A and B of the
// two-pass 3D FFT (see fft3d_fused.cu for the decomposition).
//
// k_rz (one tile per CTA) loads its whole tile, computes, then stores: with
// a 128 KiB tile only one CTA fits on an SM and HBM idles on that SM while
// it computes.  k_rz_pipe keeps the CTA resident and walks tiles
// blockIdx.x, blockIdx.x + gridDim.x, ...; the raw rows of the next tile
// are fetched with cp.async into the same shared-memory tile as soon as the
// z-FFT has read its last-stage inputs, so the fetch overlaps the last
// stage, the stores of the current tile and the tile switch.
//
// Tile layout in shared memory: block rr (residue row r*nj + k1) at
// rr*KS, z-major, X columns per z.  The radix-R step then runs in place
// (every thread reads the R values of its (z, x) pairs and writes the R
// outputs back to the same addresses), and the z-FFT works as in k_rz.
// Tiles are disjoint regions of the grid, so prefetching tile i+1 while
// tile i is stored never reads data that tile i writes.
#include "fft3d_fused.cuh"
#include "fft3d_fused_cfg.cuh"

namespace fftgb {

// At least 1024 resident threads per SM: 64 registers per thread at most.
template <int NZ, int R, int X, bool INV>
__global__ void __launch_bounds__(RzCfg<NZ, R, X>::THREADS, 1024 / RzCfg<NZ, R, X>::THREADS)
    k_rz_pipe(const FusedArgs a, long long ntiles) {
  using K = RzCfg<NZ, R, X>;
  using CZ = typename K::CZ;
  constexpr int E = K::E;
  constexpr int THREADS = K::THREADS;
  constexpr int XH = X / 2;  // 16-byte copies per row segment of a tile
  constexpr int COPIES = R * NZ * XH / THREADS;
  static_assert(X % 2 == 0 && (R * NZ * XH) % THREADS == 0, "copy split");
  extern __shared__ float2 tile[];
  pdl_enter();
  const int tid = threadIdx.x;
  const int nj = a.ny / R;
  const int xblocks = a.nx / X;
  const long long plane_pts = (long long)a.ny * a.nx;
  const long long per_b = (long long)xblocks * nj;
  const long long row_step = (long long)nj * a.nx;  // residue row r -> r+1

  auto origin = [&](long long tl) -> long long {
    const int xb = (int)(tl % xblocks);
    const int k1 = (int)((tl / xblocks) % nj);
    const long long b = tl / per_b;
    return b * NZ * plane_pts + (long long)k1 * a.nx + (long long)xb * X;
  };
  auto issue = [&](long long tl) {
    const float2 *src = a.in + origin(tl);
#pragma unroll
    for (int i = 0; i < COPIES; i++) {
      const int c = tid + i * THREADS;
      const int xp = c % XH;
      const int z = (c / XH) % NZ;
      const int rr = c / (XH * NZ);
      cp_async16(&tile[rr * K::KS + z * X + 2 * xp],
                 src + z * plane_pts + rr * row_step + 2 * xp);
    }
    cp_async_commit();
  };

  long long tl = blockIdx.x;
  if (tl < ntiles) issue(tl);
  const int x = tid % X;
  for (; tl < ntiles; tl += gridDim.x) {
    cp_async_wait_all();
    __syncthreads();  // tile tl is in shared memory

    if constexpr (R > 1) {
      // ---- radix-R over the residue rows, in place
      constexpr int ITEMS = E / R;
      constexpr int ZSTEP = THREADS / X;
      const int z0 = tid / X;
      const int k1 = (int)((tl / xblocks) % nj);
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
          const float2 w = tile[rr * K::KS + z * X + x];
          u[rr] = INV ? cswap(w) : w;
          if (rr > 0 && a.twb) u[rr] = cmul(u[rr], wr[rr]);
        }
        dft<R>(u);
#pragma unroll
        for (int k2 = 0; k2 < R; k2++) tile[k2 * K::KS + z * X + x] = u[k2];
      }
      __syncthreads();
    }

    // ---- z-FFT of column (k2, x); refill the tile after the last exchange
    const int k2 = (tid / X) % R;
    const int t = tid / (X * R);
    float2 v[E];
#pragma unroll
    for (int q = 0; q < E; q++) {
      const float2 w = tile[k2 * K::KS + in_index<CZ>(t, q) * X + x];
      v[q] = (R == 1 && INV) ? cswap(w) : w;
    }
    __syncthreads();
    const long long next = tl + gridDim.x;
    auto hook = [&]() {
      __syncthreads();  // every thread has read its last-stage inputs
      if (next < ntiles) issue(next);
    };
    stockham_h<CZ>(v, t, [k2, x](int i) -> float2 & {
      extern __shared__ float2 tile_[];
      return tile_[k2 * K::KS + i * X + x];
    }, a.tw_z, hook);
    float2 *d = a.out + origin(tl) + k2 * row_step + x;
#pragma unroll
    for (int q = 0; q < E; q++) {
      float2 w = v[q];
      if (a.scale != 1.0f) w = cscale(w, a.scale);
      d[out_index<CZ>(t, q) * plane_pts] = INV ? cswap(w) : w;
    }
  }
}

// Persistent pass A: tile (plane, r) = the NJ rows y = R*j + r of a plane,
// fetched with cp.async (each row is NX*8 contiguous bytes).  The x-FFT
// reads its inputs from the raw tile; the tile of the next (plane, r) is
// fetched once the y-FFT has read its last-stage inputs.  Pass A is out of
// place (R > 1) or works plane by plane (R == 1), so the prefetch never
// reads what the current tile writes.
template <int NX, int NJ, bool INV>
__global__ void __launch_bounds__(XyCfg<NX, NJ>::THREADS, 1024 / XyCfg<NX, NJ>::THREADS)
    k_xy_pipe(const FusedArgs a, long long ntiles) {
  using K = XyCfg<NX, NJ>;
  using CX = typename K::CX;
  using CJ = typename K::CJ;
  constexpr int E = K::E;
  constexpr int THREADS = K::THREADS;
  constexpr int XH = NX / 2;
  constexpr int COPIES = NJ * XH / THREADS;
  static_assert((NJ * XH) % THREADS == 0, "copy split");
  extern __shared__ float2 tile[];
  pdl_enter();
  const int tid = threadIdx.x;
  const int R = a.ny / NJ;

  auto issue = [&](long long tl) {
    const long long plane = tl / R;
    const int r = (int)(tl - plane * R);
    const float2 *src = a.in + (plane * a.ny + r) * NX;
#pragma unroll
    for (int i = 0; i < COPIES; i++) {
      const int c = tid + i * THREADS;
      const int j = c / XH;
      const int xp = c - j * XH;
      cp_async16(&tile[j * NX + 2 * xp], src + (long long)R * j * NX + 2 * xp);
    }
    cp_async_commit();
  };

  long long tl = blockIdx.x;
  if (tl < ntiles) issue(tl);
  for (; tl < ntiles; tl += gridDim.x) {
    const long long plane = tl / R;
    const int r = (int)(tl - plane * R);
    cp_async_wait_all();
    __syncthreads();  // raw rows of tile tl are in shared memory

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
      __syncthreads();  // every thread has read its last-stage inputs
      if (next < ntiles) issue(next);
    };
    stockham_h<CJ>(v, t, [k](int i) -> float2 & {
      extern __shared__ float2 tile_[];
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
}

namespace {
struct XyPipeEntry {
  int nx, nj;
  void (*fn[2])(const FusedArgs, long long);
  int threads, smem;
  int grid;
};

#define XYP(NX, NJ)                                                          \
  {NX, NJ, {k_xy_pipe<NX, NJ, false>, k_xy_pipe<NX, NJ, true>},              \
   XyCfg<NX, NJ>::THREADS, XyCfg<NX, NJ>::SMEM, 0}

XyPipeEntry kXyPipe[] = {
    XYP(256, 64), XYP(256, 32), XYP(128, 128), XYP(128, 64), XYP(64, 64),
    XYP(512, 32), XYP(32, 32), XYP(1024, 16), XYP(64, 16),
};

struct PipeEntry {
  int nz, r, x;
  void (*fn[2])(const FusedArgs, long long);
  int threads, smem;
  int grid;  // resident CTAs on the device (occupancy x SMs)
};

#define RZP(NZ, R, X)                                                        \
  {NZ, R, X, {k_rz_pipe<NZ, R, X, false>, k_rz_pipe<NZ, R, X, true>},        \
   RzCfg<NZ, R, X>::THREADS, RzCfg<NZ, R, X>::SMEM, 0}

PipeEntry kPipe[] = {
    RZP(256, 8, 8), RZP(256, 8, 4), RZP(256, 4, 8), RZP(256, 4, 16),
    RZP(256, 2, 32), RZP(128, 2, 16), RZP(128, 2, 32), RZP(128, 1, 32),
    RZP(128, 1, 64), RZP(64, 1, 32), RZP(64, 1, 64), RZP(32, 1, 32),
};
bool g_pipe_ready = false;
}  // namespace

cudaError_t fused_pipe_init() {
  if (g_pipe_ready) return cudaSuccess;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  for (PipeEntry &p : kPipe) {
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
  for (XyPipeEntry &p : kXyPipe) {
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
  g_pipe_ready = true;
  return cudaSuccess;
}

bool fused_xy_pipe_available(int nx, int nj) {
  for (const XyPipeEntry &p : kXyPipe)
    if (p.nx == nx && p.nj == nj) return true;
  return false;
}

cudaError_t launch_fused_xy_pipe(int nj, const FusedArgs &a, cudaStream_t s, bool pdl) {
  if (!g_pipe_ready) return cudaErrorInvalidValue;
  if (((uintptr_t)a.in & 15) || ((uintptr_t)a.out & 15))
    return cudaErrorMisalignedAddress;
  for (const XyPipeEntry &p : kXyPipe) {
    if (p.nx == a.nx && p.nj == nj) {
      if (a.ny % nj) return cudaErrorInvalidValue;
      const long long ntiles = (long long)a.nz * a.batch * (a.ny / nj);
      if (ntiles <= 0) return cudaErrorInvalidConfiguration;
      const int grid = ntiles < p.grid ? (int)ntiles : p.grid;
      return launch_k(p.fn[a.swap_io ? 1 : 0], dim3(grid), dim3(p.threads), p.smem, s, pdl,
                      a, ntiles);
    }
  }
  return cudaErrorInvalidValue;
}

bool fused_rz_pipe_available(int nz, int r, int x) {
  for (const PipeEntry &p : kPipe)
    if (p.nz == nz && p.r == r && p.x == x) return true;
  return false;
}

cudaError_t launch_fused_rz_pipe(int r, int x, const FusedArgs &a, cudaStream_t s,
                                 bool pdl) {
  if (!g_pipe_ready) return cudaErrorInvalidValue;
  // 16-byte cp.async needs 16-byte aligned rows
  if (((uintptr_t)a.in & 15) || ((uintptr_t)a.out & 15) || (a.nx & 1))
    return cudaErrorMisalignedAddress;
  for (const PipeEntry &p : kPipe) {
    if (p.nz == a.nz && p.r == r && p.x == x) {
      if (a.ny % r || a.nx % x) return cudaErrorInvalidValue;
      const long long ntiles = a.batch * (a.ny / r) * (a.nx / x);
      if (ntiles <= 0) return cudaErrorInvalidConfiguration;
      const int grid = ntiles < p.grid ? (int)ntiles : p.grid;
      return launch_k(p.fn[a.swap_io ? 1 : 0], dim3(grid), dim3(p.threads), p.smem, s, pdl,
                      a, ntiles);
    }
  }
  return cudaErrorInvalidValue;
}

}  // namespace fftgb
