// fft3d_cluster.cu - one launch per direction for 3D grids of at most 2^18
// points (2 MiB): a 16-CTA thread-block cluster holds the whole grid in its
// shared memory, so every point crosses HBM once on the way in and once on
// the way out, and the three axis FFTs run back to back in one kernel.
//
// Replaces the reference's on-chip 3D variant, which keeps the whole cube in
// BRAM (kernels/fft3d/fft3d_bram.cl:232-363, buf3D[N*N*N] at :238; driven by
// api/src/fft3d.c:30-196).
//
// CTA c of the cluster owns planes z in [c*P, (c+1)*P), P = nz/16.  Every
// axis FFT of length L = 16*T is split n = s + T*q (lane s < T holds the 16
// points q of the transform), k = k2 + 16*k1:
//   DFT16 over q in registers, twiddle W_L^(s*k2), then DFT_T over the T
//   lanes (radix-2 decimation-in-frequency butterflies by shfl.xor), after
//   which lane s holds X[k2 + 16*bitrev_T(s)] in register k2.
// So each axis touches shared memory once to read and once to write:
//   x: rows read straight from HBM, results into the CTA's planes;
//   y: columns of the CTA's own planes, in place;
//   cluster barrier (every CTA's planes complete and visible);
//   z: CTA c owns the columns y in [c*ny/16, (c+1)*ny/16) (all x); lane s
//      reads z = s + T*q from the owning CTAs' planes (distributed shared
//      memory loads) and stores the outputs straight to HBM;
//   split cluster barrier: no CTA leaves while others may still read it.
// Every CTA has read its whole input before the first cluster barrier and
// no output is stored before it, so the transform may run in place.
//
// Shared memory: point (p, y, x) of the CTA's planes sits at
// p*ny*nx + y*nx + (x ^ h), h = (((y ^ (y >> 4) ^ p) & 3) << 2) | ((x >> 4) & 3)
// (a permutation of the 16-point bank groups within a row).  With it every
// warp access of the three phases (8 rows x 4 lanes for x; 8 consecutive
// columns x 4 lanes for y and z; reads and writes) meets each 8-byte bank
// pair exactly twice for 64-point axes, the minimum for 32 x 8 bytes.
#include <cooperative_groups.h>

#include "fft_core.cuh"
#include "fft3d_cluster.cuh"

namespace cg = cooperative_groups;

namespace fftgb {

namespace {
constexpr int C3_CTAS = 16;

template <int NX, int NY, int NZ>
struct C3dCfg {
  static constexpr int P = NZ / C3_CTAS;      // planes per CTA
  static constexpr int PTS = P * NY * NX;     // points per CTA
  static constexpr int THREADS = PTS / 16;    // 16 points per thread
  static constexpr int TX = NX / 16, TY = NY / 16, TZ = NZ / 16;  // lanes per transform
  static constexpr int YC = NY / C3_CTAS;     // z phase: y rows per CTA
  static constexpr int SMEM = PTS * (int)sizeof(float2);
  static_assert(NZ % C3_CTAS == 0 && NX >= 16 && NY >= 16, "sides of 16, 32 or 64");
  static_assert(TX <= 4 && TY <= 4 && TZ <= 4, "lane DFTs of up to 4 lanes");
  static_assert(THREADS <= 1024, "one CTA of at most 1024 threads");
  static_assert(THREADS % 32 == 0 || (TX == 1 && TY == 1 && TZ == 1),
                "lane shuffles need whole warps");
};

template <int T>
__device__ __forceinline__ int brev_t(int s) {
  if constexpr (T == 4) return ((s & 1) << 1) | (s >> 1);
  return s;  // T = 1, 2
}

// Offset of point (p, y, x) in a CTA's planes (see the layout above).
template <int NY, int NX>
__device__ __forceinline__ int c3_off(int p, int y, int x) {
  const int h = ((((y ^ (y >> 4)) ^ p) & 3) << 2) | ((x >> 4) & 3);
  return (p * NY + y) * NX + (x ^ h);
}

// One axis FFT of length L = 16*T whose inputs n = s + T*q sit in register q
// of lane s (lanes of one transform are STRIDE apart within the warp).
// Afterwards lane s holds X[k2 + 16*bitrev_T(s)] in register k2.
template <int L, int STRIDE>
__device__ __forceinline__ void axis_fft(float2 (&v)[16], int s,
                                         const float2 *__restrict__ tw) {
  constexpr int T = L / 16;
  dft<16>(v);
  if constexpr (T > 1) {
#pragma unroll
    for (int k2 = 1; k2 < 16; k2++) v[k2] = cmul(v[k2], __ldg(&tw[s * k2]));
    // DFT_T over the lanes: decimation in frequency, span m = T/2, ..., 1;
    // the upper lane of a pair takes (a - b) * W_{2m}^(s mod m)
#pragma unroll
    for (int m = T / 2; m >= 1; m >>= 1) {
      const bool up = (s & m) != 0;
      const bool rot = up && m == 2 && (s & 1);  // W_4^1 = -i
#pragma unroll
      for (int q = 0; q < 16; q++) {
        float2 o;
        o.x = __shfl_xor_sync(0xffffffffu, v[q].x, m * STRIDE);
        o.y = __shfl_xor_sync(0xffffffffu, v[q].y, m * STRIDE);
        const float2 r = up ? csub(o, v[q]) : cadd(v[q], o);
        v[q] = rot ? cmul_mi(r) : r;
      }
    }
  }
}

template <int NX, int NY, int NZ, bool INV>
__global__ void __cluster_dims__(C3_CTAS, 1, 1)
    __launch_bounds__(C3dCfg<NX, NY, NZ>::THREADS, 1) k_3d_cluster(const C3dArgs a) {
  using K = C3dCfg<NX, NY, NZ>;
  constexpr int P = K::P, TX = K::TX, TY = K::TY, TZ = K::TZ, YC = K::YC;
  extern __shared__ __align__(16) float2 sm[];
  cg::cluster_group cluster = cg::this_cluster();
  const int c = (int)cluster.block_rank();
  const long long gbase = (long long)(blockIdx.x / C3_CTAS) * (NX * NY * NZ);
  const int tid = threadIdx.x;

  // ---- x: row (p, y) of the CTA's planes, lane s; inputs from HBM
  {
    const int s = tid % TX;
    const int row = tid / TX;
    const int p = row / NY, y = row % NY;
    const float2 *src = a.in + gbase + ((long long)(c * P + p) * NY + y) * NX;
    float2 v[16];
#pragma unroll
    for (int q = 0; q < 16; q++) {
      const float2 x = src[s + TX * q];
      v[q] = INV ? cswap(x) : x;
    }
    axis_fft<NX, 1>(v, s, a.tw_x);
#pragma unroll
    for (int k2 = 0; k2 < 16; k2++) sm[c3_off<NY, NX>(p, y, k2 + 16 * brev_t<TX>(s))] = v[k2];
  }
  __syncthreads();

  // ---- y: column (p, x), lane s; W consecutive columns per lane group
  {
    constexpr int W = (32 / TY) < NX ? 32 / TY : NX;
    const int xl = tid % W;
    const int s = (tid / W) % TY;
    const int grp = tid / (W * TY);
    const int x = (grp % (NX / W)) * W + xl;
    const int p = grp / (NX / W);
    float2 v[16];
#pragma unroll
    for (int q = 0; q < 16; q++) v[q] = sm[c3_off<NY, NX>(p, s + TY * q, x)];
    axis_fft<NY, W>(v, s, a.tw_y);
    // a column's rows are read and written only by its own lanes, which are
    // in this warp: every read is done once the warp is past this point
    __syncwarp();
#pragma unroll
    for (int k2 = 0; k2 < 16; k2++) sm[c3_off<NY, NX>(p, k2 + 16 * brev_t<TY>(s), x)] = v[k2];
  }
  cluster.sync();  // every CTA's planes are complete and visible cluster-wide

  // ---- z: column (y, x), y in [c*YC, (c+1)*YC); inputs from the owners
  {
    constexpr int W = (32 / TZ) < NX ? 32 / TZ : NX;
    const int xl = tid % W;
    const int s = (tid / W) % TZ;
    const int grp = tid / (W * TZ);
    const int x = (grp % (NX / W)) * W + xl;
    const int y = c * YC + grp / (NX / W);
    float2 v[16];
#pragma unroll
    for (int q = 0; q < 16; q++) {
      const int z = s + TZ * q;
      const float2 *owner = cluster.map_shared_rank(sm, z / P);
      v[q] = owner[c3_off<NY, NX>(z % P, y, x)];
    }
    // this CTA has read everything it needs from the others
    asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
    axis_fft<NZ, W>(v, s, a.tw_z);
    float2 *dst = a.out + gbase + (long long)y * NX + x;
#pragma unroll
    for (int k2 = 0; k2 < 16; k2++) {
      float2 o = v[k2];
      if (a.scale != 1.0f) o = cscale(o, a.scale);
      dst[(long long)(k2 + 16 * brev_t<TZ>(s)) * (NX * NY)] = INV ? cswap(o) : o;
    }
    // stay resident until every CTA of the cluster has read this one's planes
    asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
  }
}

struct C3dEntry {
  int nx, ny, nz;
  void (*fn[2])(const C3dArgs);  // [inverse]
  int threads, smem;
};
#define C3D(X, Y, Z)                                                    \
  {X, Y, Z, {k_3d_cluster<X, Y, Z, false>, k_3d_cluster<X, Y, Z, true>}, \
   C3dCfg<X, Y, Z>::THREADS, C3dCfg<X, Y, Z>::SMEM}
#define C3D_Z(X, Y) C3D(X, Y, 16), C3D(X, Y, 32), C3D(X, Y, 64)
#define C3D_YZ(X) C3D_Z(X, 16), C3D_Z(X, 32), C3D_Z(X, 64)
const C3dEntry kC3d[] = {C3D_YZ(16), C3D_YZ(32), C3D_YZ(64)};
bool g_c3d_ready = false;
}  // namespace

cudaError_t cluster3d_init() {
  if (g_c3d_ready) return cudaSuccess;
  for (const C3dEntry &e : kC3d)
    for (int d = 0; d < 2; d++) {
      cudaError_t r = cudaFuncSetAttribute((const void *)e.fn[d],
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, e.smem);
      // 16-CTA clusters are a non-portable size
      if (r == cudaSuccess)
        r = cudaFuncSetAttribute((const void *)e.fn[d],
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
      if (r != cudaSuccess) return r;
    }
  g_c3d_ready = true;
  return cudaSuccess;
}

static const C3dEntry *find_c3d(int nx, int ny, int nz) {
  for (const C3dEntry &e : kC3d)
    if (e.nx == nx && e.ny == ny && e.nz == nz) return &e;
  return nullptr;
}

bool cluster3d_available(int nx, int ny, int nz) { return find_c3d(nx, ny, nz) != nullptr; }

cudaError_t launch_cluster3d(int nx, int ny, int nz, const C3dArgs &a, cudaStream_t s) {
  const C3dEntry *e = find_c3d(nx, ny, nz);
  if (!g_c3d_ready || !e) return cudaErrorInvalidValue;
  const long long grid = a.batch * C3_CTAS;
  if (grid <= 0 || grid > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  e->fn[a.swap_io ? 1 : 0]<<<(unsigned)grid, e->threads, e->smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace fftgb
