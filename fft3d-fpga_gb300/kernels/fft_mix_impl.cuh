// fft_mix_impl.cuh - the mixed-radix axis kernel for lengths n = 2^a 3^b 5^c
// (n <= 8192), instantiated by fft_mix.cu (generic), fft_mix2_*.cu and
// fft_mix3_*.cu (two- and three-stage plans), fft_mix_real.cu (real-data x
// passes) and fft_mix_4s.cu (four-step passes of long 1D transforms).  One
// kernel per axis: a Stockham transform with stages of radix 16, 15, 12, 10,
// 9, 8, 6, 5, 4, 3 and 2 (the composite ones done in registers by a small
// Cooley-Tukey split).  The reference supports powers of two only; this is
// the non-power-of-two extension for the smooth lengths (any other length
// takes Bluestein's algorithm, fft_blue.cu).
//
// Stage s of radix R (NS = product of the earlier radices, m = n/R) takes,
// for every butterfly j < m with k = j mod NS, the points j + q*m (q < R),
// multiplies point q by W_n^(q*k*n/(NS*R)), applies the R-point DFT and
// writes output q to (j - k)*R + k + q*NS.  After the last stage the line is
// in natural order.  The twiddle exponent q*k*n/(NS*R) is an exact integer
// below n, so every twiddle is one entry of a FP64-generated table of n
// values.  k = j mod NS comes from a multiply-high by ceil(2^32/NS), exact
// because j*NS < 2^32 (Granlund and Montgomery, "Division by invariant
// integers using multiplication", PLDI 1994).
//
// The first stage reads its points straight from global memory and the last
// writes straight to it (both at consecutive j, so consecutive threads touch
// consecutive points of a line, or consecutive lines of a strided axis);
// the stages in between go through one shared-memory copy of the CTA's lines.
// Each thread owns butterflies t, t + T, ... of every stage (T threads per
// line; at most ceil(16/R) butterflies of radix R, one for R >= 9 in CTAs of
// up to 256 threads): it reads all of them into registers, the CTA
// synchronises, and it writes them back, so one buffer serves every stage in
// place.  The host picks the factorisation of n with the fewest stages.  The
// inverse transform is the forward one between two real/imaginary swaps.
//
// Contiguous lines (stride 1) sit one after the other in shared memory with
// one pad point per 16 (the radix-R write of the first stage goes at stride
// R); lines of a strided axis are interleaved point by point ([point][line]),
// so a warp reading one point of consecutive lines reads one run.
#pragma once

#include "fft_core.cuh"
#include "fft_mix.cuh"

namespace fftgb {

// Exact values of the radix-3 and radix-5 DFT constants (mathematical
// constants).
#define FFTGB_S3 0.86602540378443864676f   // sin(2 pi/3) = sqrt(3)/2
#define FFTGB_C5A 0.30901699437494742410f  // cos(2 pi/5)
#define FFTGB_C5B 0.80901699437494742410f  // -cos(4 pi/5)
#define FFTGB_S5A 0.95105651629515357212f  // sin(2 pi/5)
#define FFTGB_S5B 0.58778525229247312917f  // sin(4 pi/5)

template <int R>
__device__ __forceinline__ void dftm(float2 *v) {
  dft<R>(v);
}

template <>
__device__ __forceinline__ void dftm<3>(float2 *v) {
  const float2 a = v[0], t = cadd(v[1], v[2]), d = csub(v[1], v[2]);
  const float2 m = make_float2(a.x - 0.5f * t.x, a.y - 0.5f * t.y);
  const float2 r = make_float2(FFTGB_S3 * d.y, -FFTGB_S3 * d.x);  // -i sin(2pi/3) d
  v[0] = cadd(a, t);
  v[1] = cadd(m, r);
  v[2] = csub(m, r);
}

template <>
__device__ __forceinline__ void dftm<5>(float2 *v) {
  const float2 x0 = v[0];
  const float2 t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
  const float2 d1 = csub(v[1], v[4]), d2 = csub(v[2], v[3]);
  const float2 a1 = make_float2(x0.x + FFTGB_C5A * t1.x - FFTGB_C5B * t2.x,
                                x0.y + FFTGB_C5A * t1.y - FFTGB_C5B * t2.y);
  const float2 a2 = make_float2(x0.x - FFTGB_C5B * t1.x + FFTGB_C5A * t2.x,
                                x0.y - FFTGB_C5B * t1.y + FFTGB_C5A * t2.y);
  const float2 b1 = make_float2(FFTGB_S5A * d1.x + FFTGB_S5B * d2.x,
                                FFTGB_S5A * d1.y + FFTGB_S5B * d2.y);
  const float2 b2 = make_float2(FFTGB_S5B * d1.x - FFTGB_S5A * d2.x,
                                FFTGB_S5B * d1.y - FFTGB_S5A * d2.y);
  const float2 r1 = cmul_mi(b1), r2 = cmul_mi(b2);  // -i b
  v[0] = make_float2(x0.x + t1.x + t2.x, x0.y + t1.y + t2.y);
  v[1] = cadd(a1, r1);
  v[4] = csub(a1, r1);
  v[2] = cadd(a2, r2);
  v[3] = csub(a2, r2);
}

// W_N^e = e^(-2 pi i e/N) for the inner twiddles of the composite radices
// (cos and sin of 2 pi e/N in FP64, rounded to FP32).
template <int N>
__device__ __forceinline__ float2 wconst(int e);
template <>
__device__ __forceinline__ float2 wconst<6>(int e) {
  const float c[6] = {1.000000000e+00f, 5.000000000e-01f, -5.000000000e-01f, -1.000000000e+00f,
      -5.000000000e-01f, 5.000000000e-01f};
  const float s[6] = {0.000000000e+00f, 8.660254038e-01f, 8.660254038e-01f, 0.000000000e+00f,
      -8.660254038e-01f, -8.660254038e-01f};
  return make_float2(c[e], -s[e]);
}
template <>
__device__ __forceinline__ float2 wconst<9>(int e) {
  const float c[9] = {1.000000000e+00f, 7.660444431e-01f, 1.736481777e-01f, -5.000000000e-01f,
      -9.396926208e-01f, -9.396926208e-01f, -5.000000000e-01f, 1.736481777e-01f,
      7.660444431e-01f};
  const float s[9] = {0.000000000e+00f, 6.427876097e-01f, 9.848077530e-01f, 8.660254038e-01f,
      3.420201433e-01f, -3.420201433e-01f, -8.660254038e-01f, -9.848077530e-01f,
      -6.427876097e-01f};
  return make_float2(c[e], -s[e]);
}
template <>
__device__ __forceinline__ float2 wconst<10>(int e) {
  const float c[10] = {1.000000000e+00f, 8.090169944e-01f, 3.090169944e-01f, -3.090169944e-01f,
      -8.090169944e-01f, -1.000000000e+00f, -8.090169944e-01f, -3.090169944e-01f,
      3.090169944e-01f, 8.090169944e-01f};
  const float s[10] = {0.000000000e+00f, 5.877852523e-01f, 9.510565163e-01f, 9.510565163e-01f,
      5.877852523e-01f, 0.000000000e+00f, -5.877852523e-01f, -9.510565163e-01f,
      -9.510565163e-01f, -5.877852523e-01f};
  return make_float2(c[e], -s[e]);
}
template <>
__device__ __forceinline__ float2 wconst<12>(int e) {
  const float c[12] = {1.000000000e+00f, 8.660254038e-01f, 5.000000000e-01f, 0.000000000e+00f,
      -5.000000000e-01f, -8.660254038e-01f, -1.000000000e+00f, -8.660254038e-01f,
      -5.000000000e-01f, 0.000000000e+00f, 5.000000000e-01f, 8.660254038e-01f};
  const float s[12] = {0.000000000e+00f, 5.000000000e-01f, 8.660254038e-01f, 1.000000000e+00f,
      8.660254038e-01f, 5.000000000e-01f, 0.000000000e+00f, -5.000000000e-01f, -8.660254038e-01f,
      -1.000000000e+00f, -8.660254038e-01f, -5.000000000e-01f};
  return make_float2(c[e], -s[e]);
}
template <>
__device__ __forceinline__ float2 wconst<15>(int e) {
  const float c[15] = {1.000000000e+00f, 9.135454576e-01f, 6.691306064e-01f, 3.090169944e-01f,
      -1.045284633e-01f, -5.000000000e-01f, -8.090169944e-01f, -9.781476007e-01f,
      -9.781476007e-01f, -8.090169944e-01f, -5.000000000e-01f, -1.045284633e-01f,
      3.090169944e-01f, 6.691306064e-01f, 9.135454576e-01f};
  const float s[15] = {0.000000000e+00f, 4.067366431e-01f, 7.431448255e-01f, 9.510565163e-01f,
      9.945218954e-01f, 8.660254038e-01f, 5.877852523e-01f, 2.079116908e-01f, -2.079116908e-01f,
      -5.877852523e-01f, -8.660254038e-01f, -9.945218954e-01f, -9.510565163e-01f,
      -7.431448255e-01f, -4.067366431e-01f};
  return make_float2(c[e], -s[e]);
}

// Composite radix N = A*B in registers (Cooley-Tukey with n = B*n1 + n2 and
// k = k1 + A*k2): B DFTs of length A over n1, the twiddles W_N^(n2*k1), then
// A DFTs of length B over n2.  Natural order in and out.
template <int A, int B>
__device__ __forceinline__ void dft_ct(float2 *v) {
  constexpr int N = A * B;
  float2 y[B][A];
#pragma unroll
  for (int n2 = 0; n2 < B; n2++) {
#pragma unroll
    for (int n1 = 0; n1 < A; n1++) y[n2][n1] = v[B * n1 + n2];
    dftm<A>(y[n2]);
  }
#pragma unroll
  for (int n2 = 1; n2 < B; n2++)
#pragma unroll
    for (int k1 = 1; k1 < A; k1++) y[n2][k1] = cmul(y[n2][k1], wconst<N>(n2 * k1));
#pragma unroll
  for (int k1 = 0; k1 < A; k1++) {
    float2 t[B];
#pragma unroll
    for (int n2 = 0; n2 < B; n2++) t[n2] = y[n2][k1];
    dftm<B>(t);
#pragma unroll
    for (int k2 = 0; k2 < B; k2++) v[k1 + A * k2] = t[k2];
  }
}

template <>
__device__ __forceinline__ void dftm<6>(float2 *v) {
  dft_ct<3, 2>(v);
}
template <>
__device__ __forceinline__ void dftm<9>(float2 *v) {
  dft_ct<3, 3>(v);
}
template <>
__device__ __forceinline__ void dftm<10>(float2 *v) {
  dft_ct<5, 2>(v);
}
template <>
__device__ __forceinline__ void dftm<12>(float2 *v) {
  dft_ct<4, 3>(v);
}
template <>
__device__ __forceinline__ void dftm<15>(float2 *v) {
  dft_ct<5, 3>(v);
}

constexpr int MIX_EMAX = 16;      // points per thread and stage, at most
constexpr int MIX_THREADS = 512;  // threads per CTA, at most
constexpr int MIX_SMALL = 256;    // CTAs of up to this many threads: three per SM

// Butterflies of radix R per thread and stage, at most: ceil(16/R), but one
// for R >= 9 in the small CTAs (their 80-register budget).
__host__ __device__ constexpr int mix_nb(int r, bool big) {
  return (r >= 9 && !big) ? 1 : (MIX_EMAX + r - 1) / r;
}

// The real-data forms of the kernel (template parameter RL): 0 complex, 1
// R2C (the last stage stays in shared memory; an epilogue splits the packed
// transform into the n + 1 spectrum values), 2 C2R (the first stage forms
// the packed spectrum from X[k] and X[n - k] on its load).
struct MixLine {
  long long gbase;  // global index of the line's point 0 (output rows for C2R)
  long long ibase;  // C2R: global index of the line's spectrum row (n + 1 values)
  long long obase;  // four-step row pass: global index of the line's output 0
  int lcol;         // four-step column pass: the line's column j1
  int fl;           // line within the CTA
  int t;            // thread within the line
  int T;            // threads per line
  int F;            // lines per CTA
  bool ok;          // the line exists
};

template <bool STRIDED>
__device__ __forceinline__ int mix_sidx(const MixLine &L, int lp, int i) {
  return STRIDED ? i * L.F + L.fl : L.fl * lp + i + (i >> 4);
}

// One stage.  MODE 0: the first (global -> shared), 1: a middle one
// (shared -> shared), 2: the last (shared -> global), 3: the only one
// (global -> global).  RL: the real-data form (above).  EPI: the four-step
// pass the last stage stores for (MixArgs::epi; 0 a plain pass).
template <int R, int MODE, bool INV, bool STRIDED, bool BIG, int RL = 0, int EPI = 0>
__device__ __forceinline__ void mix_stage(const MixArgs &a, const MixLine &L, float2 *sm,
                                          int lp, int ns) {
  constexpr bool FIRST = MODE == 0 || MODE == 3, LAST = MODE >= 2;
  constexpr bool TO_GLOBAL = LAST && RL != 1;
  constexpr int NB = mix_nb(R, BIG);
  const int n = a.n, m = n / R;
  const int tws = n / (ns * R);
  const unsigned magic = ns > 1 ? 0xffffffffu / (unsigned)ns + 1u : 0u;
  const long long gstride = STRIDED ? a.inner : 1;
  float2 v[NB][R];
#pragma unroll
  for (int b = 0; b < NB; b++) {
    const int j = L.t + b * L.T;
    if (j < m) {
      if (FIRST && RL == 2) {  // packed spectrum (X[i] + conj X[n-i]) + i W^-i (X[i] - conj X[n-i])
        const float2 *X = a.in + L.ibase;
#pragma unroll
        for (int q = 0; q < R; q++) {
          const int i = j + q * m;
          float2 z = make_float2(0.f, 0.f);
          if (L.ok) {
            const float2 xk = X[i], xm = X[n - i];
            const float2 sp = make_float2(xk.x + xm.x, xk.y - xm.y);
            const float2 d = make_float2(xk.x - xm.x, xk.y + xm.y);
            const float2 w = __ldg(&a.wn[i]);
            const float2 dw = cmul(d, make_float2(w.x, -w.y));
            z = make_float2(sp.x - dw.y, sp.y + dw.x);
          }
          v[b][q] = INV ? cswap(z) : z;
        }
      } else if (FIRST) {
        const float2 *src = a.in + L.gbase + (long long)j * gstride;
#pragma unroll
        for (int q = 0; q < R; q++) {
          float2 x = make_float2(0.f, 0.f);
          if (L.ok) x = src[(long long)(q * m) * gstride];
          v[b][q] = INV ? cswap(x) : x;
        }
      } else {
        const int k = j - (int)__umulhi((unsigned)j, magic) * ns;
#pragma unroll
        for (int q = 0; q < R; q++) v[b][q] = sm[mix_sidx<STRIDED>(L, lp, j + q * m)];
        const int kt = k * tws;
#pragma unroll
        for (int q = 1; q < R; q++) v[b][q] = cmul(v[b][q], __ldg(&a.w[q * kt]));
      }
      dftm<R>(v[b]);
    }
  }
  // every read of this stage lands before any write of it (one buffer)
  if (MODE == 1 || (MODE == 2 && RL == 1)) __syncthreads();
#pragma unroll
  for (int b = 0; b < NB; b++) {
    const int j = L.t + b * L.T;
    if (j < m) {
      const int k = FIRST ? 0 : j - (int)__umulhi((unsigned)j, magic) * ns;
      const int d = (j - k) * R + k;
      if (TO_GLOBAL) {
        if (L.ok) {
          const long long ostride = EPI == 2 ? a.ep_n2 : gstride;
          float2 *dst = a.out + (EPI == 2 ? L.obase : L.gbase) + (long long)d * ostride;
#pragma unroll
          for (int q = 0; q < R; q++) {
            float2 y = INV ? cswap(v[b][q]) : v[b][q];
            if (EPI == 1) {  // W_N^(j1 k2), conjugate for the inverse
              const int e = L.lcol * (d + q * ns);
              float2 w = cmul(__ldg(&a.tw_hi[e >> 12]), __ldg(&a.tw_lo[e & 4095]));
              if (INV) w.y = -w.y;
              y = cmul(y, w);
            }
            if (a.scale != 1.0f) y = cscale(y, a.scale);
            dst[(long long)(q * ns) * ostride] = y;
          }
        }
      } else {
#pragma unroll
        for (int q = 0; q < R; q++) sm[mix_sidx<STRIDED>(L, lp, d + q * ns)] = v[b][q];
      }
    }
  }
  if (!TO_GLOBAL) __syncthreads();
}

#define FFTGB_MIX_RADICES(X) X(16) X(15) X(12) X(10) X(9) X(8) X(6) X(5) X(4) X(3) X(2)

// A radix's position in the stage order above, and back.
__host__ __device__ constexpr int mix_rank(int r) {
  return r == 16 ? 0 : r == 15 ? 1 : r == 12 ? 2 : r == 10 ? 3 : r == 9 ? 4 : r == 8 ? 5
         : r == 6 ? 6 : r == 5 ? 7 : r == 4 ? 8 : r == 3 ? 9 : r == 2 ? 10 : -1;
}
__host__ __device__ constexpr int mix_radix(int rank) {
  return rank == 0 ? 16 : rank == 1 ? 15 : rank == 2 ? 12 : rank == 3 ? 10 : rank == 4 ? 9
         : rank == 5 ? 8 : rank == 6 ? 6 : rank == 7 ? 5 : rank == 8 ? 4 : rank == 9 ? 3 : 2;
}

template <int MODE, bool INV, bool STRIDED, bool BIG, int RL, int EPI = 0>
__device__ __forceinline__ void mix_stage_r(int rank, const MixArgs &a, const MixLine &L,
                                            float2 *sm, int lp, int ns) {
  switch (rank) {
#define FFTGB_MIX_CASE(R) \
  case mix_rank(R): mix_stage<R, MODE, INV, STRIDED, BIG, RL, EPI>(a, L, sm, lp, ns); break;
    FFTGB_MIX_RADICES(FFTGB_MIX_CASE)
#undef FFTGB_MIX_CASE
  }
}

// NT: the most threads a CTA of the instantiation has; CTAs of up to 256
// threads run three to an SM (80 registers), larger ones one (128).
// The thread's line and position in it (F lines of T threads per CTA).
template <bool STRIDED, int EPI = 0>
__device__ __forceinline__ MixLine mix_line(const MixArgs &a, int F, int T, long long *line) {
  const int tid = threadIdx.x;
  MixLine L;
  L.F = F;
  L.T = T;
  L.fl = STRIDED ? tid % F : tid / T;
  L.t = STRIDED ? tid / F : tid % T;
  *line = (long long)blockIdx.x * F + L.fl;
  L.ok = *line < a.nlines;
  L.gbase = 0;
  L.ibase = 0;
  L.obase = 0;
  L.lcol = 0;
  if (L.ok) {
    const long long o = *line / a.inner;
    L.gbase = o * a.n * a.inner + (*line - o * a.inner);
    L.ibase = *line * (a.n + 1);  // C2R rows of n + 1 (inner = 1)
    if (EPI == 1) L.lcol = (int)(*line - o * a.inner);
    if (EPI == 2) {
      const long long t = *line / a.ep_n2;
      L.obase = t * a.ep_N + (*line - t * a.ep_n2);
    }
  }
  return L;
}

// R2C epilogue: X[k] = E[k] + W_2n^k O[k], k = 0..n, from the packed
// transform Z of the line in shared memory.
__device__ __forceinline__ void mix_r2c_split(const MixArgs &a, const MixLine &L,
                                              const float2 *smem, int lp, long long line) {
  if (!L.ok) return;
  const int n = a.n;
  float2 *dst = a.out + line * (n + 1);
  for (int k = L.t; k <= n; k += L.T) {
    const float2 zk = smem[mix_sidx<false>(L, lp, k == n ? 0 : k)];
    const float2 zm = smem[mix_sidx<false>(L, lp, k == 0 ? 0 : n - k)];
    const float2 e = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
    const float2 o = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
    float2 x = cadd(e, cmul(__ldg(&a.wn[k]), o));
    if (a.scale != 1.0f) x = cscale(x, a.scale);
    dst[k] = x;
  }
}

// Two-stage plans (radix R0 then R1) with only those two stage bodies in the
// kernel: the generic kernel, which holds every radix, runs the same stages
// about 14 % slower.
template <int R0, int R1, bool INV, bool STRIDED, int RL = 0, int EPI = 0>
__global__ void __launch_bounds__(MIX_SMALL, 3) k_mix2(const MixArgs a, int F, int T) {
  extern __shared__ float2 smem[];
  long long line;
  const MixLine L = mix_line<STRIDED, EPI>(a, F, T, &line);
  const int lp = a.n + (a.n >> 4) + 1;
  mix_stage<R0, 0, INV, STRIDED, false, RL, EPI>(a, L, smem, lp, 1);
  mix_stage<R1, 2, INV, STRIDED, false, RL, EPI>(a, L, smem, lp, R0);
  if constexpr (RL == 1) mix_r2c_split(a, L, smem, lp, line);
}

// The pairs (R0, R1) of the two-stage plans, k_mix2's instantiations
// (kernels/fft_mix2_*.cu: a third each, and the power-of-two pairs beside the
// third part).
#define FFTGB_MIX2_PAIRS_A(X) \
  X(5, 5) X(6, 3) X(6, 6) X(8, 5) X(9, 3) X(9, 6) X(9, 9) X(10, 2) X(10, 5) X(10, 10)
#define FFTGB_MIX2_PAIRS_B(X) \
  X(12, 2) X(12, 6) X(12, 9) X(12, 12) X(15, 2) X(15, 3) X(15, 4) X(15, 5) X(15, 6) X(15, 8)
#define FFTGB_MIX2_PAIRS_C(X) \
  X(15, 9) X(15, 10) X(15, 12) X(15, 15) X(16, 3) X(16, 5) X(16, 6) X(16, 10) X(16, 12) X(16, 15)
// power-of-two factors of the four-step passes (32, 64, 128, 256)
#define FFTGB_MIX2_PAIRS_D(X) X(8, 4) X(16, 4) X(16, 8) X(16, 16)

// Three-stage plans (R0, R1, R2), likewise: the 66 radix triples the
// factorisation picks for 256 < n <= 4096 in the 256-thread CTAs.
template <int R0, int R1, int R2, bool INV, bool STRIDED, int RL = 0, int EPI = 0>
__global__ void __launch_bounds__(MIX_SMALL, 3) k_mix3(const MixArgs a, int F, int T) {
  extern __shared__ float2 smem[];
  long long line;
  const MixLine L = mix_line<STRIDED, EPI>(a, F, T, &line);
  const int lp = a.n + (a.n >> 4) + 1;
  mix_stage<R0, 0, INV, STRIDED, false, RL, EPI>(a, L, smem, lp, 1);
  mix_stage<R1, 1, INV, STRIDED, false, RL, EPI>(a, L, smem, lp, R0);
  mix_stage<R2, 2, INV, STRIDED, false, RL, EPI>(a, L, smem, lp, R0 * R1);
  if constexpr (RL == 1) mix_r2c_split(a, L, smem, lp, line);
}

// k_mix3's instantiations (kernels/fft_mix3_*.cu, a sixth each).
#define FFTGB_MIX3_TRIPLES_D(X) \
  X(5, 5, 5) X(9, 9, 9) X(12, 9, 9) X(15, 6, 3) X(15, 9, 9) X(15, 15, 2) X(15, 15, 9) \
  X(16, 6, 3) X(16, 10, 5) X(16, 15, 5) X(16, 16, 3)
#define FFTGB_MIX3_TRIPLES_E(X) \
  X(6, 6, 6) X(10, 5, 5) X(12, 12, 3) X(15, 6, 6) X(15, 10, 5) X(15, 15, 3) X(15, 15, 10) \
  X(16, 6, 5) X(16, 10, 10) X(16, 15, 6) X(16, 16, 5)
#define FFTGB_MIX3_TRIPLES_F(X) \
  X(8, 5, 5) X(10, 10, 5) X(12, 12, 6) X(15, 8, 3) X(15, 10, 10) X(15, 15, 4) X(15, 15, 12) \
  X(16, 6, 6) X(16, 12, 6) X(16, 15, 8) X(16, 16, 6)
#define FFTGB_MIX3_TRIPLES_G(X) \
  X(9, 9, 2) X(10, 10, 10) X(12, 12, 12) X(15, 8, 5) X(15, 12, 6) X(15, 15, 5) X(15, 15, 15) \
  X(16, 8, 3) X(16, 12, 12) X(16, 15, 10) X(16, 16, 10)
#define FFTGB_MIX3_TRIPLES_H(X) \
  X(9, 9, 3) X(12, 9, 3) X(15, 5, 4) X(15, 9, 3) X(15, 12, 9) X(15, 15, 6) X(16, 5, 4) \
  X(16, 8, 5) X(16, 15, 3) X(16, 15, 12) X(16, 16, 12)
#define FFTGB_MIX3_TRIPLES_I(X) \
  X(9, 9, 6) X(12, 9, 6) X(15, 5, 5) X(15, 9, 6) X(15, 12, 12) X(15, 15, 8) X(16, 5, 5) \
  X(16, 9, 9) X(16, 15, 4) X(16, 15, 15) X(16, 16, 15)

typedef void (*MixFn)(const MixArgs, int, int);
// Entry [rank R0][rank R1][inverse][strided] (rank: position in 16, 15, 12,
// 10, 9, 8, 6, 5, 4, 3, 2) of each two-stage kernel; filled by the three
// translation units.
typedef MixFn MixPairTable[11][11][2][2];
// [rank R0][rank R1][epi - 1][inverse]: the four-step passes' two-stage kernels
typedef MixFn MixPairEpiTable[11][11][2][2];
void mix2_fill_epi_a(MixPairEpiTable &t);
void mix2_fill_epi_b(MixPairEpiTable &t);
void mix2_fill_epi_c(MixPairEpiTable &t);
// [epi - 1][inverse][more than 256 threads]: their generic kernels
typedef MixFn MixEpiTable[2][2][2];
void mix_fill_epi(MixEpiTable &t);
// [rank R0][rank R1][c2r]: the real-data forms of the two-stage kernels
typedef MixFn MixPairRealTable[11][11][2];
void mix2_fill_real_a(MixPairRealTable &t);
void mix2_fill_real_b(MixPairRealTable &t);
void mix2_fill_real_c(MixPairRealTable &t);
void mix2_fill_a(MixPairTable &t);
void mix2_fill_b(MixPairTable &t);
void mix2_fill_c(MixPairTable &t);
typedef MixFn MixTripleTable[11][11][11][2][2];
typedef MixFn MixTripleRealTable[11][11][11][2];  // [ranks][c2r]: real-data forms
typedef MixFn MixTripleEpiTable[11][11][11][2][2];  // [ranks][epi - 1][inverse]: four-step
void mix3_fill_d(MixTripleTable &t);
void mix3_fill_real_d(MixTripleRealTable &t);
void mix3_fill_epi_d(MixTripleEpiTable &t);
void mix3_fill_e(MixTripleTable &t);
void mix3_fill_real_e(MixTripleRealTable &t);
void mix3_fill_epi_e(MixTripleEpiTable &t);
void mix3_fill_f(MixTripleTable &t);
void mix3_fill_real_f(MixTripleRealTable &t);
void mix3_fill_epi_f(MixTripleEpiTable &t);
void mix3_fill_g(MixTripleTable &t);
void mix3_fill_real_g(MixTripleRealTable &t);
void mix3_fill_epi_g(MixTripleEpiTable &t);
void mix3_fill_h(MixTripleTable &t);
void mix3_fill_real_h(MixTripleRealTable &t);
void mix3_fill_epi_h(MixTripleEpiTable &t);
void mix3_fill_i(MixTripleTable &t);
void mix3_fill_real_i(MixTripleRealTable &t);
void mix3_fill_epi_i(MixTripleEpiTable &t);

#define FFTGB_MIX3_FILL(R0, R1, R2)                                                       \
  t[mix_rank(R0)][mix_rank(R1)][mix_rank(R2)][0][0] = k_mix3<R0, R1, R2, false, false>;   \
  t[mix_rank(R0)][mix_rank(R1)][mix_rank(R2)][1][0] = k_mix3<R0, R1, R2, true, false>;    \
  t[mix_rank(R0)][mix_rank(R1)][mix_rank(R2)][0][1] = k_mix3<R0, R1, R2, false, true>;    \
  t[mix_rank(R0)][mix_rank(R1)][mix_rank(R2)][1][1] = k_mix3<R0, R1, R2, true, true>;
#define FFTGB_MIX3_FILL_EPI(R0, R1, R2)                                                   \
  t[mix_rank(R0)][mix_rank(R1)][mix_rank(R2)][0][0] = k_mix3<R0, R1, R2, false, true, 0, 1>;  \
  t[mix_rank(R0)][mix_rank(R1)][mix_rank(R2)][0][1] = k_mix3<R0, R1, R2, true, true, 0, 1>;   \
  t[mix_rank(R0)][mix_rank(R1)][mix_rank(R2)][1][0] = k_mix3<R0, R1, R2, false, false, 0, 2>; \
  t[mix_rank(R0)][mix_rank(R1)][mix_rank(R2)][1][1] = k_mix3<R0, R1, R2, true, false, 0, 2>;
#define FFTGB_MIX3_FILL_REAL(R0, R1, R2)                                                  \
  t[mix_rank(R0)][mix_rank(R1)][mix_rank(R2)][0] = k_mix3<R0, R1, R2, false, false, 1>;  \
  t[mix_rank(R0)][mix_rank(R1)][mix_rank(R2)][1] = k_mix3<R0, R1, R2, true, false, 2>;
#define FFTGB_MIX2_FILL_REAL(R0, R1)                                     \
  t[mix_rank(R0)][mix_rank(R1)][0] = k_mix2<R0, R1, false, false, 1>;   \
  t[mix_rank(R0)][mix_rank(R1)][1] = k_mix2<R0, R1, true, false, 2>;
#define FFTGB_MIX2_FILL_EPI(R0, R1)                                               \
  t[mix_rank(R0)][mix_rank(R1)][0][0] = k_mix2<R0, R1, false, true, 0, 1>;        \
  t[mix_rank(R0)][mix_rank(R1)][0][1] = k_mix2<R0, R1, true, true, 0, 1>;         \
  t[mix_rank(R0)][mix_rank(R1)][1][0] = k_mix2<R0, R1, false, false, 0, 2>;       \
  t[mix_rank(R0)][mix_rank(R1)][1][1] = k_mix2<R0, R1, true, false, 0, 2>;
#define FFTGB_MIX2_FILL(R0, R1)                                                   \
  t[mix_rank(R0)][mix_rank(R1)][0][0] = k_mix2<R0, R1, false, false>;             \
  t[mix_rank(R0)][mix_rank(R1)][1][0] = k_mix2<R0, R1, true, false>;              \
  t[mix_rank(R0)][mix_rank(R1)][0][1] = k_mix2<R0, R1, false, true>;              \
  t[mix_rank(R0)][mix_rank(R1)][1][1] = k_mix2<R0, R1, true, true>;

template <bool INV, bool STRIDED, int NT, int RL = 0, int EPI = 0>
__global__ void __launch_bounds__(NT, NT <= MIX_SMALL ? 3 : 1) k_mix(const MixArgs a, int F, int T) {
  constexpr bool BIG = NT > MIX_SMALL;
  extern __shared__ float2 smem[];
  long long line;
  const MixLine L = mix_line<STRIDED, EPI>(a, F, T, &line);
  const int lp = a.n + (a.n >> 4) + 1;  // contiguous layout: padded line pitch
  const int nst = a.nst;
  const unsigned long long code = a.rcode;
  const int rk0 = (int)(code & 15);
  if (nst == 1) {
    mix_stage_r<RL == 1 ? 0 : 3, INV, STRIDED, BIG, RL, EPI>(rk0, a, L, smem, lp, 1);
  } else {
    mix_stage_r<0, INV, STRIDED, BIG, RL, EPI>(rk0, a, L, smem, lp, 1);
    // The middle stages, one loop per radix (the radices come grouped in the
    // order 16, 15, 12, 10, 9, 8, 6, 5, 4, 3, 2): each loop holds one stage
    // body, so what the compiler hoists out of it belongs to that radix alone.
    int ns = mix_radix(rk0), st = 1;
#define FFTGB_MIX_MID(R)                                                          \
  for (; st < nst - 1 && (int)((code >> (4 * st)) & 15) == mix_rank(R); st++) {  \
    mix_stage<R, 1, INV, STRIDED, BIG, RL>(a, L, smem, lp, ns);   \
    ns *= R;                                                      \
  }
    FFTGB_MIX_RADICES(FFTGB_MIX_MID)
#undef FFTGB_MIX_MID
    mix_stage_r<2, INV, STRIDED, BIG, RL, EPI>((int)((code >> (4 * (nst - 1))) & 15), a, L,
                                               smem, lp, ns);
  }
  if constexpr (RL == 1) mix_r2c_split(a, L, smem, lp, line);
}

// Launch shape of a k_mix pass (host side, kernels/fft_mix.cu).
struct MixShape {
  int F, T;         // lines per CTA, threads per line
  bool big;         // the 512-thread instantiation
  long long grid;
  size_t smem;
  unsigned long long rcode;  // MixArgs::rcode of the radices
};
cudaError_t mix_shape(const MixArgs &a, int lines_per_cta, bool real, MixShape *sh);
// the real-data instantiations (kernels/fft_mix_real.cu)
cudaError_t mix_real_init();

}  // namespace fftgb
