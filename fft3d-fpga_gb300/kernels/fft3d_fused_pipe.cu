// fft3d_fused_pipe.cu - persistent, software-pipelined form of pass B of the
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
#pragma unroll
      for (int m = 0; m < ITEMS; m++) {
        const int z = z0 + m * ZSTEP;
        float2 u[R];
#pragma unroll
        for (int rr = 0; rr < R; rr++) {
          const float2 w = tile[rr * K::KS + z * X + x];
          u[rr] = INV ? cswap(w) : w;
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

namespace {
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
  g_pipe_ready = true;
  return cudaSuccess;
}

bool fused_rz_pipe_available(int nz, int r, int x) {
  for (const PipeEntry &p : kPipe)
    if (p.nz == nz && p.r == r && p.x == x) return true;
  return false;
}

cudaError_t launch_fused_rz_pipe(int r, int x, const FusedArgs &a, cudaStream_t s) {
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
      p.fn[a.swap_io ? 1 : 0]<<<grid, p.threads, p.smem, s>>>(a, ntiles);
      return cudaGetLastError();
    }
  }
  return cudaErrorInvalidValue;
}

}  // namespace fftgb
