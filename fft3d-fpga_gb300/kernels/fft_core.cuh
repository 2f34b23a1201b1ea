// fft_core.cuh - register/shared-memory building blocks of the sm_103a FFT
// kernels: radix-2/4/8/16 DFTs in registers and a cooperative Stockham
// (self-sorting) FFT whose middle stages exchange data through shared memory.
//
// Replaces the reference's radix-2^2 feed-forward engine
// (kernels/common/fft_8.cl:61-346).  Conventions kept: forward sign -
// (fft_8.cl:240), inverse = forward applied between a real/imaginary swap
// on input and output (fft_8.cl:276-278, 341-343), which conjugates the whole
// linear map and therefore gives the unnormalised inverse.  Twiddles come
// from tables generated on the host in FP64 and rounded once to FP32.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fftgb {

__host__ __device__ constexpr int ilog2c(long long v) {
  return v <= 1 ? 0 : 1 + ilog2c(v >> 1);
}

// ----------------------------------------------------------------- complex
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
  return make_float2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
  return make_float2(a.x - b.x, a.y - b.y);
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * (-i)
__device__ __forceinline__ float2 cmul_mi(float2 a) {
  return make_float2(a.y, -a.x);
}
__device__ __forceinline__ float2 cswap(float2 a) {
  return make_float2(a.y, a.x);
}
__device__ __forceinline__ float2 cscale(float2 a, float s) {
  return make_float2(a.x * s, a.y * s);
}

// Exact values of cos/sin at multiples of pi/8 used inside the radix-8/16
// butterflies (mathematical constants).
#define FFTGB_C8 0.70710678118654752440f   // cos(pi/4)
#define FFTGB_C16 0.92387953251128675613f  // cos(pi/8)
#define FFTGB_S16 0.38268343236508977173f  // sin(pi/8)

// ------------------------------------------------------- radix-R DFTs
// In-place forward DFT of v[0..R-1], natural order in and out.
template <int R>
__device__ __forceinline__ void dft(float2 *v);

template <>
__device__ __forceinline__ void dft<1>(float2 *) {}

template <>
__device__ __forceinline__ void dft<2>(float2 *v) {
  float2 a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

__device__ __forceinline__ void dft4_io(float2 &x0, float2 &x1, float2 &x2,
                                        float2 &x3) {
  float2 s02 = cadd(x0, x2), d02 = csub(x0, x2);
  float2 s13 = cadd(x1, x3), d13 = cmul_mi(csub(x1, x3));
  x0 = cadd(s02, s13);
  x2 = csub(s02, s13);
  x1 = cadd(d02, d13);
  x3 = csub(d02, d13);
}

template <>
__device__ __forceinline__ void dft<4>(float2 *v) {
  dft4_io(v[0], v[1], v[2], v[3]);
}

// multiply by W8^1 = (1 - i)/sqrt(2)
__device__ __forceinline__ float2 mul_w8_1(float2 a) {
  return make_float2((a.x + a.y) * FFTGB_C8, (a.y - a.x) * FFTGB_C8);
}
// multiply by W8^3 = (-1 - i)/sqrt(2)
__device__ __forceinline__ float2 mul_w8_3(float2 a) {
  return make_float2((a.y - a.x) * FFTGB_C8, -(a.x + a.y) * FFTGB_C8);
}

template <>
__device__ __forceinline__ void dft<8>(float2 *v) {
  // radix-2 decimation in time over two radix-4 halves
  float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  float2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  dft4_io(e0, e1, e2, e3);
  dft4_io(o0, o1, o2, o3);
  o1 = mul_w8_1(o1);
  o2 = cmul_mi(o2);
  o3 = mul_w8_3(o3);
  v[0] = cadd(e0, o0);
  v[4] = csub(e0, o0);
  v[1] = cadd(e1, o1);
  v[5] = csub(e1, o1);
  v[2] = cadd(e2, o2);
  v[6] = csub(e2, o2);
  v[3] = cadd(e3, o3);
  v[7] = csub(e3, o3);
}

// W16^1 = cos(pi/8) - i sin(pi/8)
__device__ __forceinline__ float2 mul_w16_1(float2 a) {
  return make_float2(a.x * FFTGB_C16 + a.y * FFTGB_S16,
                     a.y * FFTGB_C16 - a.x * FFTGB_S16);
}
// W16^3 = sin(pi/8) - i cos(pi/8)
__device__ __forceinline__ float2 mul_w16_3(float2 a) {
  return make_float2(a.x * FFTGB_S16 + a.y * FFTGB_C16,
                     a.y * FFTGB_S16 - a.x * FFTGB_C16);
}
// W16^9 = -W16^1
__device__ __forceinline__ float2 mul_w16_9(float2 a) {
  return make_float2(-(a.x * FFTGB_C16 + a.y * FFTGB_S16),
                     a.x * FFTGB_S16 - a.y * FFTGB_C16);
}

template <>
__device__ __forceinline__ void dft<16>(float2 *v) {
  // 4 x 4 decomposition: n = 4*n1 + n2, k = k1 + 4*k2.
  // columns: DFT4 over n1 for each n2 -> y[n2 + 4*k1]
  dft4_io(v[0], v[4], v[8], v[12]);
  dft4_io(v[1], v[5], v[9], v[13]);
  dft4_io(v[2], v[6], v[10], v[14]);
  dft4_io(v[3], v[7], v[11], v[15]);
  // twiddles W16^(n2*k1)
  v[5] = mul_w16_1(v[5]);
  v[9] = mul_w8_1(v[9]);    // W16^2
  v[13] = mul_w16_3(v[13]);
  v[6] = mul_w8_1(v[6]);    // W16^2
  v[10] = cmul_mi(v[10]);   // W16^4
  v[14] = mul_w8_3(v[14]);  // W16^6
  v[7] = mul_w16_3(v[7]);
  v[11] = mul_w8_3(v[11]);  // W16^6
  v[15] = mul_w16_9(v[15]);
  // rows: DFT4 over n2 for each k1 -> X[k1 + 4*k2] in v[4*k1 + k2]
  dft4_io(v[0], v[1], v[2], v[3]);
  dft4_io(v[4], v[5], v[6], v[7]);
  dft4_io(v[8], v[9], v[10], v[11]);
  dft4_io(v[12], v[13], v[14], v[15]);
  // transpose the 4x4 register block into natural order
  float2 t;
  t = v[1]; v[1] = v[4]; v[4] = t;
  t = v[2]; v[2] = v[8]; v[8] = t;
  t = v[3]; v[3] = v[12]; v[12] = t;
  t = v[6]; v[6] = v[9]; v[9] = t;
  t = v[7]; v[7] = v[13]; v[13] = t;
  t = v[11]; v[11] = v[14]; v[14] = t;
}

// -------------------------------------------------- Stockham configuration
// A Stockham plan of length L with E points held per thread: T = L/E threads
// per transform, stage radices E, E, ..., and a last stage of the remaining
// radix.  Stage s reads element j + k*L/R and writes (j/NS)*NS*R + j%NS +
// k*NS for the butterflies j = t + m*T a thread owns.
__host__ __device__ constexpr int default_e(int L) {
  return (L <= 16) ? L : ((L == 32 || L == 64) ? 8 : 16);
}

template <int L_, int E_>
struct Stock {
  static constexpr int L = L_;
  static constexpr int LOG = ilog2c(L_);
  static constexpr int E = (E_ < L_) ? E_ : L_;
  static constexpr int T = L / E;
  static constexpr int LOGE = ilog2c(E);
  static constexpr int NSTG = (LOG + LOGE - 1) / LOGE;
  // radix of stage s
  __host__ __device__ static constexpr int radix(int s) {
    return (s < NSTG - 1) ? E : (1 << (LOG - LOGE * (NSTG - 1)));
  }
  // product of the radices of stages before s
  __host__ __device__ static constexpr int ns(int s) { return 1 << (LOGE * s); }
  static constexpr int RLAST = radix(NSTG - 1);
  // Twiddle table of this plan: one block per stage s >= 1 holding
  // W_{NS*R}^(jr*k) at [k][jr] (R x NS entries), so the threads of a warp,
  // which differ in jr, read consecutive entries.  Blocks are back to back.
  __host__ __device__ static constexpr int stage_off(int s) {
    return s <= 1 ? 0 : stage_off(s - 1) + radix(s - 1) * ns(s - 1);
  }
  static constexpr int TABLE = stage_off(NSTG);
};

template <int L>
using Cfg = Stock<L, default_e(L)>;

// Shared-memory swizzle inside one transform: XOR the low 4 bits of the
// index with a fold of the higher bits.  Keeps Stockham scatter stores and
// bit-reversed reads free of 8-byte bank conflicts.
__device__ __forceinline__ int swz(int i) {
  return i ^ (((i >> 4) ^ (i >> 8) ^ (i >> 12)) & 15);
}

// Radix-16 butterflies in registers (the default; the tensor-core form in
// fft_tc.cu supplies its own functor with the same call).
struct PlainR16 {
  __device__ __forceinline__ void operator()(float2 *v) { dft<16>(v); }
};

// One Stockham stage on registers: twiddle by W_{NS*R}^{(j mod NS) k}
// (from the plan's stage table `tw`, see Stock::stage_off), then DFT_R, for
// the E/R butterflies j = t + m*T this thread owns.  Radix-16 butterflies go
// through `r16`.
template <class C, int S, class F16>
__device__ __forceinline__ void stage_compute(float2 (&v)[C::E], int t,
                                              const float2 *__restrict__ tw,
                                              F16 &r16) {
  constexpr int E = C::E, T = C::T;
  constexpr int R = C::radix(S), NS = C::ns(S);
  constexpr int NB = E / R;
  constexpr int OFF = C::stage_off(S);
#pragma unroll
  for (int m = 0; m < NB; m++) {
    if (NS > 1) {
      const int jr = (t + m * T) & (NS - 1);
#pragma unroll
      for (int k = 1; k < R; k++) {
        const float2 w = __ldg(&tw[OFF + k * NS + jr]);
        v[m * R + k] = cmul(v[m * R + k], w);
      }
    }
    if constexpr (R == 16)
      r16(&v[m * R]);
    else
      dft<R>(&v[m * R]);
  }
}

template <class C, int S>
__device__ __forceinline__ void stage_compute(float2 (&v)[C::E], int t,
                                              const float2 *__restrict__ tw) {
  PlainR16 r16;
  stage_compute<C, S>(v, t, tw, r16);
}

// Index (within the transform) that register v[m*R + k] is read from in
// stage S, and where stage S writes it.
template <class C, int S>
__device__ __forceinline__ int stage_in_index(int t, int m, int k) {
  constexpr int R = C::radix(S);
  return t + m * C::T + k * (C::L / R);
}

template <class C, int S>
__device__ __forceinline__ int stage_out_index(int t, int m, int k) {
  constexpr int R = C::radix(S), NS = C::ns(S);
  const int j = t + m * C::T;
  return (j / NS) * NS * R + (j & (NS - 1)) + k * NS;
}

// Index the last stage leaves register v[q] at (natural order).
template <class C>
__device__ __forceinline__ int out_index(int t, int q) {
  constexpr int R = C::RLAST;
  return stage_in_index<C, C::NSTG - 1>(t, q / R, q % R);
}

// Input index of register q for stage 0.
template <class C>
__device__ __forceinline__ int in_index(int t, int q) {
  constexpr int R0 = C::radix(0);
  return stage_in_index<C, 0>(t, q / R0, q % R0);
}

// Barrier between the exchange steps of one transform.  MODE 0: the whole
// CTA; 1: the calling warp (the transform's threads and shared-memory slice
// lie within one warp); 2: named barrier `id` over the transform's COUNT
// threads (whole warps that only this transform's exchange involves).
template <int MODE, int COUNT = 0>
__device__ __forceinline__ void xchg_sync(int id) {
  if constexpr (MODE == 1) {
    __syncwarp();
  } else if constexpr (MODE == 2) {
    static_assert(COUNT % 32 == 0, "named barriers count whole warps");
    asm volatile("bar.sync %0, %1;\n" ::"r"(id), "n"(COUNT) : "memory");
  } else {
    __syncthreads();
  }
}

// Middle and last stages: read registers from shared memory, compute, and
// (for non-last stages) write back.  `sm(i)` returns a reference into the
// calling transform's shared-memory slice.  Every thread that the barrier
// MODE covers must call this (it contains the barriers).
template <class C, int S, int MODE, class SM, class F16>
__device__ __forceinline__ void stockham_rest_b(float2 (&v)[C::E], int t, SM sm,
                                                const float2 *__restrict__ tw,
                                                F16 &r16, int bar_id) {
  constexpr int E = C::E, NSTG = C::NSTG;
  if constexpr (S < NSTG) {
    constexpr int R = C::radix(S);
#pragma unroll
    for (int q = 0; q < E; q++) v[q] = sm(stage_in_index<C, S>(t, q / R, q % R));
    if constexpr (S < NSTG - 1) xchg_sync<MODE, C::T>(bar_id);
    stage_compute<C, S>(v, t, tw, r16);
    if constexpr (S < NSTG - 1) {
#pragma unroll
      for (int q = 0; q < E; q++) sm(stage_out_index<C, S>(t, q / R, q % R)) = v[q];
      xchg_sync<MODE, C::T>(bar_id);
      stockham_rest_b<C, S + 1, MODE>(v, t, sm, tw, r16, bar_id);
    }
  }
}

template <class C, int S, class SM, class F16>
__device__ __forceinline__ void stockham_rest(float2 (&v)[C::E], int t, SM sm,
                                              const float2 *__restrict__ tw,
                                              F16 &r16) {
  stockham_rest_b<C, S, 0>(v, t, sm, tw, r16, 0);
}

template <class C, int MODE, class SM, class F16>
__device__ __forceinline__ void stockham_b(float2 (&v)[C::E], int t, SM sm,
                                           const float2 *__restrict__ tw,
                                           F16 &r16, int bar_id) {
  constexpr int E = C::E, NSTG = C::NSTG, R0 = C::radix(0);
  stage_compute<C, 0>(v, t, tw, r16);
  if constexpr (NSTG > 1) {
#pragma unroll
    for (int q = 0; q < E; q++) sm(stage_out_index<C, 0>(t, q / R0, q % R0)) = v[q];
    xchg_sync<MODE, C::T>(bar_id);
    stockham_rest_b<C, 1, MODE>(v, t, sm, tw, r16, bar_id);
  }
}

// Full transform: registers v hold the stage-0 inputs (v[q] = x[in_index]),
// leaves the outputs in v (v[q] = X[out_index(t, q)]).  With more than one
// stage, the first exchange writes `sm` without a barrier first: callers
// that reuse `sm` must synchronise before calling.
template <class C, class SM, class F16>
__device__ __forceinline__ void stockham(float2 (&v)[C::E], int t, SM sm,
                                         const float2 *__restrict__ tw,
                                         F16 &r16) {
  stockham_b<C, 0>(v, t, sm, tw, r16, 0);
}

template <class C, class SM>
__device__ __forceinline__ void stockham(float2 (&v)[C::E], int t, SM sm,
                                         const float2 *__restrict__ tw) {
  PlainR16 r16;
  stockham<C>(v, t, sm, tw, r16);
}

// stockham() for the rows of a row tile of ROWS rows: row f is transformed
// by threads f*T .. f*T + T - 1 and only they touch its shared-memory slice,
// so its exchange barriers need not involve the other rows: a warp barrier
// when T divides 32, a named barrier (id 1 + f, T threads) when a row spans
// whole warps and the tile has at most 15 rows (ids 1-15; 0 is the CTA's),
// the CTA barrier otherwise.
template <class C, int ROWS>
constexpr int row_sync_mode() {
  return 32 % C::T == 0 ? 1 : (C::T % 32 == 0 && ROWS <= 15) ? 2 : 0;
}
template <class C, int ROWS>
__device__ __forceinline__ void row_sync(int row) {
  xchg_sync<row_sync_mode<C, ROWS>(), C::T>(1 + row);
}
template <class C, int ROWS, class SM>
__device__ __forceinline__ void stockham_row(float2 (&v)[C::E], int t, SM sm,
                                             const float2 *__restrict__ tw, int row) {
  PlainR16 r16;
  stockham_b<C, row_sync_mode<C, ROWS>()>(v, t, sm, tw, r16, 1 + row);
}

// As stockham(), but calls hook() once every register has been read from
// shared memory for the last time (before the last stage's arithmetic; for a
// single-stage transform, before its arithmetic), so
// a caller can start refilling the shared-memory tile while the last stage
// and its stores run.  hook() is called by every thread; it must contain
// the barrier that orders the other threads' last reads before new writes.
template <class C, int S, class SM, class H>
__device__ __forceinline__ void stockham_rest_h(float2 (&v)[C::E], int t, SM sm,
                                                const float2 *__restrict__ tw,
                                                H &hook) {
  constexpr int E = C::E, NSTG = C::NSTG;
  constexpr int R = C::radix(S);
#pragma unroll
  for (int q = 0; q < E; q++) v[q] = sm(stage_in_index<C, S>(t, q / R, q % R));
  if constexpr (S < NSTG - 1) {
    __syncthreads();
    stage_compute<C, S>(v, t, tw);
#pragma unroll
    for (int q = 0; q < E; q++) sm(stage_out_index<C, S>(t, q / R, q % R)) = v[q];
    __syncthreads();
    stockham_rest_h<C, S + 1>(v, t, sm, tw, hook);
  } else {
    hook();
    stage_compute<C, S>(v, t, tw);
  }
}

template <class C, class SM, class H>
__device__ __forceinline__ void stockham_h(float2 (&v)[C::E], int t, SM sm,
                                           const float2 *__restrict__ tw, H &hook) {
  constexpr int E = C::E, R0 = C::radix(0);
  if constexpr (C::NSTG == 1) {  // no exchange: the inputs are in registers
    hook();
    stage_compute<C, 0>(v, t, tw);
  } else {
    stage_compute<C, 0>(v, t, tw);
#pragma unroll
    for (int q = 0; q < E; q++) sm(stage_out_index<C, 0>(t, q / R0, q % R0)) = v[q];
    __syncthreads();
    stockham_rest_h<C, 1>(v, t, sm, tw, hook);
  }
}

// Ampere-style asynchronous global -> shared copies (16 bytes, L2 only):
// each thread waits for its own copies, a barrier then publishes them.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// Programmatic dependent launch.  A kernel launched by launch_k(..., pdl =
// true) may be scheduled while the previous kernel of its stream is still
// finishing; pdl_enter() blocks until that kernel has completed and its
// memory is visible, so it must run before the kernel's first global access.
// It then lets this kernel's own dependents launch (all of this grid's CTAs
// are running by the time the last one passes here).  Without the launch
// attribute both instructions return at once.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}

// Launches fn<<<grid, block, smem, s>>>(args...), with programmatic stream
// serialisation when pdl is set (fn must call pdl_enter() first).
template <typename... P, typename... A>
inline cudaError_t launch_k(void (*fn)(P...), dim3 grid, dim3 block, size_t smem,
                            cudaStream_t s, bool pdl, A... args) {
  if (!pdl) {
    fn<<<grid, block, smem, s>>>(args...);
    return cudaGetLastError();
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, fn, args...);
}

// W_N^e from a two-level FP64-generated table: lo[e & mask] * hi[e >> bits].
__device__ __forceinline__ float2 twiddle2(const float2 *__restrict__ lo,
                                           const float2 *__restrict__ hi,
                                           int bits, long long e) {
  const float2 a = __ldg(&lo[e & ((1LL << bits) - 1)]);
  const float2 b = __ldg(&hi[e >> bits]);
  return cmul(a, b);
}

// w[q] = W^(cc * i(q)) for the indexes i(q) = t + m*T + k*(L/R), q = m*R + k,
// of the stage-0 inputs (OUT false, R = radix(0)) or of the last stage's
// outputs (OUT true, R = RLAST) of thread t, W from the two-level table.
// With R a multiple of 4 the four registers of a run share m and their
// index grows by L/R, so W is geometric there: one table read per run plus
// the step W^(cc*L/R), at most 3 chained roundings; otherwise every factor
// is read.  The reads are scattered over the table (lanes differ in cc), so
// the chain cuts the read wavefronts about threefold.
template <class C, bool OUT>
__device__ __forceinline__ void tw4_factors(float2 (&w)[C::E], int t, long long cc,
                                            const float2 *__restrict__ lo,
                                            const float2 *__restrict__ hi, int bits) {
  constexpr int R = OUT ? C::RLAST : C::radix(0);
  if constexpr (R % 4 == 0) {
    const float2 step = twiddle2(lo, hi, bits, cc * (C::L / R));
#pragma unroll
    for (int q = 0; q < C::E; q++) {
      const int i = OUT ? out_index<C>(t, q) : in_index<C>(t, q);
      if (q % 4 == 0)
        w[q] = twiddle2(lo, hi, bits, cc * i);
      else
        w[q] = cmul(w[q - 1], step);
    }
  } else {
#pragma unroll
    for (int q = 0; q < C::E; q++)
      w[q] = twiddle2(lo, hi, bits, cc * (OUT ? out_index<C>(t, q) : in_index<C>(t, q)));
  }
}

template <class C, bool OUT>
__device__ __forceinline__ void tw4_mul(float2 (&v)[C::E], int t, long long cc,
                                        const float2 *__restrict__ lo,
                                        const float2 *__restrict__ hi, int bits) {
  float2 w[C::E];
  tw4_factors<C, OUT>(w, t, cc, lo, hi, bits);
#pragma unroll
  for (int q = 0; q < C::E; q++) v[q] = cmul(v[q], w[q]);
}

__device__ __forceinline__ unsigned bitrev_n(unsigned x, int bits) {
  return bits == 0 ? 0u : (__brev(x) >> (32 - bits));
}

}  // namespace fftgb
