// fft_pass.cu - generic axis passes of the sm_103a FFT library.
//
// k_rows<L>: FFTs of length L along the contiguous axis.  Replaces the
//   reference's fetch + fft1d / fft3da stages (kernels/fft1d/fft1d.cl:140-252,
//   kernels/fft3d/fft3d_ddr.cl:22-114): the stage-0 loads come straight from
//   HBM (consecutive threads read consecutive points) and the last stage
//   stores straight to HBM, so only the middle Stockham stages touch shared
//   memory.  The bit-reversed order of the 1D ABI (fft_8.cl:28-30) is made by
//   bouncing the last stage through shared memory so HBM stores stay
//   coalesced.
//
// k_cols<L, W>: FFTs of length L along a strided axis for W adjacent
//   columns per CTA (consecutive threads own consecutive columns, so every
//   HBM access is a W*8-byte contiguous run).  Replaces the reference's
//   transpose / transpose3D / fft3db / fft3dc stages
//   (kernels/fft3d/fft3d_ddr.cl:116-416), which move the y and z axes
//   through on-chip and DDR transposes; here the strided axis is read in
//   place and no transpose pass exists.  Optionally applies the four-step
//   twiddle and writes a transposed layout (large 1D transforms).
#include "fft_core.cuh"
#include "fft_pass.cuh"

namespace fftgb {

template <int L>
struct RowsCfg {
  static constexpr int THREADS = (L >= 256) ? 512 : 256;
  static constexpr int F = THREADS / Cfg<L>::T;  // rows per CTA
  static constexpr int SMEM = THREADS * Cfg<L>::E * (int)sizeof(float2);
  // out_mode 4 stages the CTA's outputs as [L][F + 1]; it needs a warp to
  // span whole rows of that stage (F divides 32) and runs of F >= 8 points
  static constexpr bool TRANSPOSE = F >= 8 && F <= 32;
  static constexpr int SMEM_T = L * (F + 1) * (int)sizeof(float2);
};

template <int L>
struct ColsCfg {
  static constexpr int T = Cfg<L>::T;
  static constexpr int W = (L <= 16)    ? 256
                           : (L <= 32)  ? 64
                           : (L <= 128) ? 64
                           : (L <= 256) ? 32
                           : (L <= 1024) ? 16
                           : (L <= 2048) ? 8
                                         : 4;
  static constexpr int THREADS = W * T;
  static constexpr int WP = W + 1;
  static constexpr int SMEM = L * WP * (int)sizeof(float2);
};

template <int L, bool INV>
__global__ void __launch_bounds__(RowsCfg<L>::THREADS, RowsCfg<L>::THREADS == 512 ? 2 : 1)
    k_rows(const RowsArgs a) {
  using C = Cfg<L>;
  constexpr int T = C::T, E = C::E, F = RowsCfg<L>::F;
  extern __shared__ float2 smem[];
  pdl_enter();
  const int tid = threadIdx.x;
  const int fl = tid / T;
  const int t = tid - fl * T;
  const long long row = (long long)blockIdx.x * F + fl;
  const bool ok = row < a.nrows;
  const float2 *src = a.in + row * L;

  float2 v[E];
#pragma unroll
  for (int q = 0; q < E; q++) {
    int idx = in_index<C>(t, q);
    if (a.in_mode == 1) idx = (int)bitrev_n((unsigned)idx, C::LOG);
    float2 x = ok ? src[idx] : make_float2(0.f, 0.f);
    v[q] = INV ? cswap(x) : x;
  }

  float2 *mysm = smem + fl * L;
  auto sm = [mysm](int i) -> float2 & { return mysm[swz(i)]; };
  stockham_row<C, F>(v, t, sm, a.tw, fl);

  if (a.scale != 1.0f) {
#pragma unroll
    for (int q = 0; q < E; q++) v[q] = cscale(v[q], a.scale);
  }

  if (a.out_mode == 0 || a.out_mode == 3) {
    long long orow = row;
    if (a.out_mode == 3) {
      // row (b, z, y) of the grids [b][nz][ny] -> (b, y/8, z, y%8)
      const int lyz = a.blk_lny + a.blk_lnz;
      const long long b = row >> lyz;
      const long long z = (row >> a.blk_lny) & ((1LL << a.blk_lnz) - 1);
      const long long y = row & ((1LL << a.blk_lny) - 1);
      orow = ((((b << (a.blk_lny - 3)) + (y >> 3)) << a.blk_lnz | z) << 3) | (y & 7);
    }
    float2 *dst = a.out + orow * L;
    if (ok) {
#pragma unroll
      for (int q = 0; q < E; q++) {
        const float2 x = v[q];
        dst[out_index<C>(t, q)] = INV ? cswap(x) : x;
      }
    }
  } else if (a.out_mode == 4) {
    if constexpr (RowsCfg<L>::TRANSPOSE) {
      // four-step transpose: row (b, k2) of transforms of 2^rows_log rows
      // puts element k at b*L*2^rows_log + k*2^rows_log + k2.  The CTA's F
      // rows are consecutive k2 of one transform, staged in shared memory
      // as [k][F] (padded to F + 1: the reads below are conflict-free), so
      // every warp stores 32 / F runs of F points instead of scattering.
      constexpr int THREADS = RowsCfg<L>::THREADS;
      constexpr int KPW = 32 / F;  // values of k per warp store
      __syncthreads();  // every row's exchange slice read before the stage overwrites it
#pragma unroll
      for (int q = 0; q < E; q++)
        smem[out_index<C>(t, q) * (F + 1) + fl] = INV ? cswap(v[q]) : v[q];
      __syncthreads();
      const long long lr = 1LL << a.rows_log;
      const long long row0 = (long long)blockIdx.x * F;
      float2 *dst = a.out + (row0 >> a.rows_log) * lr * L + (row0 & (lr - 1));
      const int lane = tid & 31;
      const int r = lane % F;
      if (row0 + r < a.nrows) {
#pragma unroll 4
        for (int k = (tid >> 5) * KPW + lane / F; k < L; k += (THREADS / 32) * KPW)
          dst[(long long)k * lr + r] = smem[k * (F + 1) + r];
      }
    }
  } else {
    // bit-reversed order within the row, through shared memory
    if (C::NSTG > 1) row_sync<C, F>(fl);
#pragma unroll
    for (int q = 0; q < E; q++) sm(out_index<C>(t, q)) = v[q];
    row_sync<C, F>(fl);
    long long orow = row;
    if (a.out_mode == 2) {
      const long long mask = (1LL << a.rows_log) - 1;
      orow = (row & ~mask) | (long long)bitrev_n((unsigned)(row & mask), a.rows_log);
    }
    float2 *dst = a.out + orow * L;
    if (ok) {
#pragma unroll
      for (int q = 0; q < E; q++) {
        const int p = t + q * T;
        const float2 x = sm((int)bitrev_n((unsigned)p, C::LOG));
        dst[p] = INV ? cswap(x) : x;
      }
    }
  }
}

template <int L, bool INV>
__global__ void __launch_bounds__(ColsCfg<L>::THREADS, ColsCfg<L>::THREADS == 512 ? 2 : 1)
    k_cols(const ColsArgs a) {
  using C = Cfg<L>;
  constexpr int E = C::E, W = ColsCfg<L>::W, WP = ColsCfg<L>::WP;
  constexpr int THREADS = ColsCfg<L>::THREADS;
  extern __shared__ float2 smem[];
  pdl_enter();
  const int tid = threadIdx.x;
  const int t = tid / W;
  const int fl = tid - t * W;
  const long long col0 = (long long)blockIdx.x * W;
  const long long col = col0 + fl;
  const bool ok = col < a.ncols;
  // 32-bit division where the column numbers allow (a 64-bit division per
  // thread is a long instruction sequence in these issue-bound passes)
  long long o, c;
  if (a.ncols < (1LL << 32)) {
    const unsigned q = (unsigned)col / (unsigned)a.inner;
    o = q;
    c = (long long)((unsigned)col - q * (unsigned)a.inner);
  } else {
    o = col / a.inner;
    c = col - o * a.inner;
  }
  const long long base = o * (long long)L * a.inner + c;

  float2 v[E];
#pragma unroll
  for (int q = 0; q < E; q++) {
    const long long idx = in_index<C>(t, q);
    float2 x = ok ? a.in[base + idx * a.inner] : make_float2(0.f, 0.f);
    v[q] = INV ? cswap(x) : x;
  }
  if (a.tw_in && a.tw4_lo != nullptr)  // W^((c >> tw_shift)*n) on the inputs n
    tw4_mul<C, false>(v, t, c >> a.tw_shift, a.tw4_lo, a.tw4_hi, a.tw4_bits);

  auto sm = [fl](int i) -> float2 & {
    extern __shared__ float2 smem_[];
    return smem_[i * WP + fl];
  };
  stockham<C>(v, t, sm, a.tw);

  if (a.tw4_lo != nullptr && !a.tw_in)  // W^(c*k) on the outputs k
    tw4_mul<C, true>(v, t, c, a.tw4_lo, a.tw4_hi, a.tw4_bits);
  if (a.scale != 1.0f) {
#pragma unroll
    for (int q = 0; q < E; q++) v[q] = cscale(v[q], a.scale);
  }

  if (a.out_mode == 0) {
    if (ok) {
#pragma unroll
      for (int q = 0; q < E; q++) {
        const long long idx = out_index<C>(t, q);
        const float2 x = v[q];
        a.out[base + idx * a.inner] = INV ? cswap(x) : x;
      }
    }
  } else {
    if (C::NSTG > 1) __syncthreads();
#pragma unroll
    for (int q = 0; q < E; q++) sm(out_index<C>(t, q)) = v[q];
    __syncthreads();
    float2 *dst = a.out + col0 * L;
#pragma unroll
    for (int q = 0; q < E; q++) {
      const int p = tid + q * THREADS;
      const int f = p / L;
      const int k = p - f * L;
      if (col0 + f < a.ncols) {
        const float2 x = smem[k * WP + f];
        dst[p] = INV ? cswap(x) : x;
      }
    }
  }
}

// out[b*n + j] = in[b*n + bitrev(j)]: undoes the 1D ABI's bit-reversed order
// (used by the adjoint of bit-reversed plans above 4096 points).
__global__ void k_bitrev_gather(const float2 *__restrict__ in,
                                float2 *__restrict__ out, long long n,
                                int log_n, long long total) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const long long b = i >> log_n;
  const long long j = i & (n - 1);
  out[i] = in[b * n + bitrev_n((unsigned)j, log_n)];
}

cudaError_t launch_bitrev_gather(const float2 *in, float2 *out, long long n,
                                 int log_n, long long count, cudaStream_t s) {
  const long long total = n * count;
  const long long grid = (total + 255) / 256;
  if (grid <= 0 || grid > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  k_bitrev_gather<<<(unsigned)grid, 256, 0, s>>>(in, out, n, log_n, total);
  return cudaGetLastError();
}

// ------------------------------------------------------------ dispatch
namespace {
typedef void (*RowsFn)(const RowsArgs);
typedef void (*ColsFn)(const ColsArgs);

constexpr int MAXLOG = 12;
// [log2 L][inverse]
RowsFn g_rows[MAXLOG + 1][2];
ColsFn g_cols[MAXLOG + 1][2];
int g_rows_smem[MAXLOG + 1], g_rows_thr[MAXLOG + 1], g_rows_f[MAXLOG + 1];
int g_rows_smem_t[MAXLOG + 1];  // out_mode 4 (0: not supported)
int g_cols_smem[MAXLOG + 1], g_cols_thr[MAXLOG + 1], g_cols_w[MAXLOG + 1];
bool g_ready = false;

template <int LOG>
struct Tab {
  static constexpr int L = 1 << LOG;
  static void fill() {
    g_rows[LOG][0] = k_rows<L, false>;
    g_rows[LOG][1] = k_rows<L, true>;
    g_cols[LOG][0] = k_cols<L, false>;
    g_cols[LOG][1] = k_cols<L, true>;
    g_rows_smem[LOG] = RowsCfg<L>::SMEM;
    g_rows_thr[LOG] = RowsCfg<L>::THREADS;
    g_rows_f[LOG] = RowsCfg<L>::F;
    g_rows_smem_t[LOG] = RowsCfg<L>::TRANSPOSE ? RowsCfg<L>::SMEM_T : 0;
    g_cols_smem[LOG] = ColsCfg<L>::SMEM;
    g_cols_thr[LOG] = ColsCfg<L>::THREADS;
    g_cols_w[LOG] = ColsCfg<L>::W;
    Tab<LOG - 1>::fill();
  }
};
template <>
struct Tab<0> {
  static void fill() {}
};

cudaError_t set_attributes() {
  Tab<MAXLOG>::fill();
  for (int l = 1; l <= MAXLOG; l++) {
    for (int d = 0; d < 2; d++) {
      cudaError_t e = cudaFuncSetAttribute(
          (const void *)g_rows[l][d], cudaFuncAttributeMaxDynamicSharedMemorySize,
          g_rows_smem_t[l] > g_rows_smem[l] ? g_rows_smem_t[l] : g_rows_smem[l]);
      if (e != cudaSuccess) return e;
      e = cudaFuncSetAttribute((const void *)g_cols[l][d],
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               g_cols_smem[l]);
      if (e != cudaSuccess) return e;
    }
  }
  return cudaSuccess;
}

cudaError_t do_launch_rows(int log_l, const RowsArgs &a, cudaStream_t s, bool pdl = false) {
  const long long f = g_rows_f[log_l];
  const long long grid = (a.nrows + f - 1) / f;
  if (grid <= 0 || grid > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  int smem = g_rows_smem[log_l];
  if (a.out_mode == 4) {
    // whole CTAs of rows within one transform
    if (!g_rows_smem_t[log_l] || a.rows_log < 0 || a.rows_log > 30 ||
        (1LL << a.rows_log) % f || a.nrows % (1LL << a.rows_log))
      return cudaErrorInvalidValue;
    if (g_rows_smem_t[log_l] > smem) smem = g_rows_smem_t[log_l];
  }
  return launch_k(g_rows[log_l][a.swap_io ? 1 : 0], dim3((unsigned)grid),
                  dim3(g_rows_thr[log_l]), smem, s, pdl, a);
}

cudaError_t do_launch_cols(int log_l, const ColsArgs &a, cudaStream_t s, bool pdl = false) {
  const long long w = g_cols_w[log_l];
  const long long grid = (a.ncols + w - 1) / w;
  if (grid <= 0 || grid > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  return launch_k(g_cols[log_l][a.swap_io ? 1 : 0], dim3((unsigned)grid),
                  dim3(g_cols_thr[log_l]), g_cols_smem[log_l], s, pdl, a);
}
}  // namespace

cudaError_t pass_kernels_init() {
  if (g_ready) return cudaSuccess;
  cudaError_t e = set_attributes();
  if (e == cudaSuccess) g_ready = true;
  return e;
}

cudaError_t pass_kernels_set_attributes_current_device() {
  return set_attributes();
}

cudaError_t launch_rows_on(int log_l, const RowsArgs &a, cudaStream_t s) {
  if (log_l < 1 || log_l > MAXLOG || g_rows[log_l][0] == nullptr)
    return cudaErrorInvalidValue;
  return do_launch_rows(log_l, a, s);
}

cudaError_t launch_cols_on(int log_l, const ColsArgs &a, cudaStream_t s) {
  if (log_l < 1 || log_l > MAXLOG || g_cols[log_l][0] == nullptr)
    return cudaErrorInvalidValue;
  return do_launch_cols(log_l, a, s);
}

int rows_threads(int log_l) { return g_rows_thr[log_l]; }

bool rows_transposed_supported(int log_l, int rows_log) {
  if (log_l < 1 || log_l > MAXLOG || !g_ready || !g_rows_smem_t[log_l]) return false;
  return rows_log >= 0 && rows_log <= 30 && (1LL << rows_log) % g_rows_f[log_l] == 0;
}
int cols_threads(int log_l) { return g_cols_thr[log_l]; }

cudaError_t launch_rows(int log_l, const RowsArgs &a, cudaStream_t s, bool pdl) {
  if (log_l < 1 || log_l > MAXLOG || !g_ready) return cudaErrorInvalidValue;
  return do_launch_rows(log_l, a, s, pdl);
}

cudaError_t launch_cols(int log_l, const ColsArgs &a, cudaStream_t s, bool pdl) {
  if (log_l < 1 || log_l > MAXLOG || !g_ready) return cudaErrorInvalidValue;
  return do_launch_cols(log_l, a, s, pdl);
}

}  // namespace fftgb
