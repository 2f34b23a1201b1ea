// fft_blue.cu - FFTs of any length n <= 2048 along one axis (Bluestein's
// chirp-z algorithm), one kernel per axis.  The reference supports powers
// of two only; this is the non-power-of-two extension.
//
// With w[m] = e^(-i pi m^2 / n) (FP64-generated, m^2 taken mod 2n) and
// nk = (n^2 + k^2 - (k-n)^2) / 2, the forward DFT is
//   X[k] = w[k] * sum_m (x[m] w[m]) conj(w[k - m]),
// a cyclic convolution of length M (the power of two >= 2n - 1) with the
// chirp filter b (b[m] = conj w[m] for |m| < n, wrapped mod M, else 0).
// Each line is loaded (zero-padded to M and multiplied by w), transformed
// with an M-point Stockham FFT, multiplied by H = DFT_M(b) / M (FP64-
// generated on the host), inverse transformed (real/imaginary swap around
// the forward FFT), multiplied by w and stored.  The inverse transform uses
// conj(w) and conj(H[-k]).  Everything between the load and the store stays
// in registers and shared memory.
//
// Lines of the contiguous axis (stride 1) are mapped one line per group of
// T threads (consecutive threads read consecutive points); lines of a
// strided axis are mapped one line per thread column (consecutive threads
// read consecutive lines, which are adjacent in memory).
#include "fft_core.cuh"
#include "fft_blue.cuh"

namespace fftgb {

template <int M>
struct BlueCfg {
  using C = Cfg<M>;
  static constexpr int THREADS = (M >= 256) ? 512 : 256;
  static constexpr int F = THREADS / C::T;  // lines per CTA
  static constexpr int FP = F + 1;          // strided layout: padded line stride
  static constexpr int SMEM_ROWS = F * M * (int)sizeof(float2);
  static constexpr int SMEM_COLS = M * FP * (int)sizeof(float2);
};

template <int M, bool INV, bool STRIDED>
__global__ void __launch_bounds__(BlueCfg<M>::THREADS, 1)
    k_blue(const BlueArgs a) {
  using C = Cfg<M>;
  using K = BlueCfg<M>;
  constexpr int T = C::T, E = C::E, F = K::F, FP = K::FP;
  extern __shared__ float2 smem[];
  const int tid = threadIdx.x;
  const int fl = STRIDED ? tid % F : tid / T;
  const int t = STRIDED ? tid / F : tid % T;
  const long long line = (long long)blockIdx.x * F + fl;
  const bool ok = line < a.nlines;
  const long long o = line / a.inner;
  const long long base = o * a.n * a.inner + (line - o * a.inner);
  auto sm = [fl](int i) -> float2 & {
    extern __shared__ float2 s_[];
    return STRIDED ? s_[i * FP + fl] : s_[fl * M + swz(i)];
  };
  auto chirp = [&](int m) -> float2 {
    const float2 w = __ldg(&a.w[m]);
    return INV ? make_float2(w.x, -w.y) : w;
  };

  // load, zero-pad, multiply by the chirp
  float2 v[E];
#pragma unroll
  for (int q = 0; q < E; q++) {
    const int m = in_index<C>(t, q);
    float2 x = make_float2(0.f, 0.f);
    if (ok && m < a.n) x = cmul(a.in[base + (long long)m * a.inner], chirp(m));
    v[q] = x;
  }
  stockham<C>(v, t, sm, a.tw);
  // multiply by the filter spectrum (1/M folded in)
#pragma unroll
  for (int q = 0; q < E; q++) {
    const int k = out_index<C>(t, q);
    float2 h;
    if (INV) {
      const float2 g = __ldg(&a.H[(M - k) & (M - 1)]);
      h = make_float2(g.x, -g.y);
    } else {
      h = __ldg(&a.H[k]);
    }
    v[q] = cmul(v[q], h);
  }
  // back to the input order of the next transform
  __syncthreads();
#pragma unroll
  for (int q = 0; q < E; q++) sm(out_index<C>(t, q)) = v[q];
  __syncthreads();
#pragma unroll
  for (int q = 0; q < E; q++) v[q] = cswap(sm(in_index<C>(t, q)));
  __syncthreads();
  // inverse M-point transform through the real/imaginary swap
  stockham<C>(v, t, sm, a.tw);
  if (!ok) return;
#pragma unroll
  for (int q = 0; q < E; q++) {
    const int k = out_index<C>(t, q);
    if (k < a.n) {
      float2 y = cmul(cswap(v[q]), chirp(k));
      if (a.scale != 1.0f) y = cscale(y, a.scale);
      a.out[base + (long long)k * a.inner] = y;
    }
  }
}

namespace {
typedef void (*BlueFn)(const BlueArgs);
constexpr int MAXLOG = 12;
BlueFn g_blue[MAXLOG + 1][2][2];  // [log M][inverse][strided]
int g_thr[MAXLOG + 1], g_f[MAXLOG + 1], g_smem[MAXLOG + 1][2];
bool g_blue_ready = false;

template <int LOG>
struct BTab {
  static constexpr int M = 1 << LOG;
  static void fill() {
    g_blue[LOG][0][0] = k_blue<M, false, false>;
    g_blue[LOG][1][0] = k_blue<M, true, false>;
    g_blue[LOG][0][1] = k_blue<M, false, true>;
    g_blue[LOG][1][1] = k_blue<M, true, true>;
    g_thr[LOG] = BlueCfg<M>::THREADS;
    g_f[LOG] = BlueCfg<M>::F;
    g_smem[LOG][0] = BlueCfg<M>::SMEM_ROWS;
    g_smem[LOG][1] = BlueCfg<M>::SMEM_COLS;
    BTab<LOG - 1>::fill();
  }
};
template <>
struct BTab<1> {
  static void fill() {}
};
}  // namespace

cudaError_t blue_kernels_init() {
  if (g_blue_ready) return cudaSuccess;
  BTab<MAXLOG>::fill();
  for (int l = 2; l <= MAXLOG; l++)
    for (int d = 0; d < 2; d++)
      for (int st = 0; st < 2; st++) {
        const cudaError_t e = cudaFuncSetAttribute(
            (const void *)g_blue[l][d][st], cudaFuncAttributeMaxDynamicSharedMemorySize,
            g_smem[l][st]);
        if (e != cudaSuccess) return e;
      }
  g_blue_ready = true;
  return cudaSuccess;
}

int blue_length(int n) {
  int m = 4;
  while (m < 2 * n - 1) m <<= 1;
  return m;
}

cudaError_t launch_blue(int log_m, int inverse, const BlueArgs &a, cudaStream_t s) {
  if (!g_blue_ready || log_m < 2 || log_m > MAXLOG || a.n < 2 || (1 << log_m) < 2 * a.n - 1)
    return cudaErrorInvalidValue;
  const int st = a.inner > 1 ? 1 : 0;
  const long long grid = (a.nlines + g_f[log_m] - 1) / g_f[log_m];
  if (grid <= 0 || grid > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  g_blue[log_m][inverse ? 1 : 0][st]<<<(unsigned)grid, g_thr[log_m], g_smem[log_m][st], s>>>(a);
  return cudaGetLastError();
}

}  // namespace fftgb
