/*
 * fftfpga_ext.h - additions to the FFTFPGA C ABI (no counterpart in the
 * reference's api/include/fftfpga/fftfpga.h unless a line says otherwise).
 *
 * Device-pointer plans for callers that keep data resident in HBM (no host
 * copy per call), explicit CUDA streams, natural-order 1D output, adjoint
 * transforms, ragged batches of 3D grids in one persistent launch, and the
 * tensor-core split-precision mode.  Only plain C types cross this boundary:
 * device buffers and streams are passed as `void *` (a CUDA device pointer
 * and a cudaStream_t; NULL is the CUDA default stream).
 *
 * Conventions are those of fftfpga.h: forward sign -, inverse unnormalised,
 * grids row-major with x fastest and batches contiguous.
 */
#ifndef FFTFPGA_EXT_H
#define FFTFPGA_EXT_H

#include <stddef.h>

#include "fftfpga.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes of every fftgb_* call. */
#define FFTGB_OK 0
#define FFTGB_EINVAL (-1)   /* bad argument (NULL, not a power of two, ...) */
#define FFTGB_ENODEV (-2)   /* no usable CUDA device */
#define FFTGB_ENOMEM (-3)   /* device or host allocation failed */
#define FFTGB_ECUDA (-4)    /* a CUDA call or kernel launch failed */
#define FFTGB_EUNSUP (-5)   /* size/mode combination not supported */
#define FFTGB_ETIMEOUT (-6) /* a bounded device wait gave up (ragged batch) */

/* Plan flags. */
#define FFTGB_ORDER_NATURAL 0x0u /* 1D output in natural order (default) */
#define FFTGB_ORDER_BITREV 0x1u  /* 1D output bit-reversed per block, the
                                    fftfpgaf_c2c_1d order */
#define FFTGB_PREC_FP32 0x00u     /* plain FP32 kernels (default) */
#define FFTGB_PREC_TC_FP16 0x10u  /* radix-16 sub-stages as split FP16
                                     (hi+lo) tensor-core GEMMs, FP32 acc. */
#define FFTGB_PREC_TC_BF16 0x20u  /* same with a 3-way BF16 split */
#define FFTGB_PREC_MASK 0xf0u

typedef struct fftgb_plan_s *fftgb_plan;

/* Plans for `batch` contiguous transforms.  nx is the fastest (contiguous)
 * axis.  Axis lengths: powers of two (up to 4096 per axis where some other
 * axis is not a power of two), 2^a 3^b 5^c up to 8192 (1D: up to 2^24), any
 * other length up to 2048; the lengths that are not powers of two take FP32
 * and the natural order only. */
int fftgb_plan_1d(fftgb_plan *plan, unsigned n, unsigned batch, unsigned flags);
int fftgb_plan_2d(fftgb_plan *plan, unsigned nx, unsigned ny, unsigned batch,
                  unsigned flags);
int fftgb_plan_3d(fftgb_plan *plan, unsigned nx, unsigned ny, unsigned nz,
                  unsigned batch, unsigned flags);
void fftgb_plan_destroy(fftgb_plan plan);

/* Number of complex points one execution reads (and writes). */
size_t fftgb_plan_points(fftgb_plan plan);

/* Number of kernel launches one execution makes (for launch accounting). */
int fftgb_plan_launches(fftgb_plan plan);

/* 1 if d_in == d_out is allowed for this plan. */
int fftgb_plan_inplace_ok(fftgb_plan plan);

/*
 * Execute on device buffers, asynchronously on `stream`.  d_in and d_out
 * are device pointers to fftgb_plan_points() float2 values each.  They may
 * be equal only when fftgb_plan_inplace_ok() says so; partial overlap is an
 * error.  `inverse` != 0 runs the unnormalised inverse.  `scale` multiplies
 * every output (1.0f: none).
 */
int fftgb_exec(fftgb_plan plan, const void *d_in, void *d_out, int inverse,
               float scale, void *stream);

/*
 * Adjoint (conjugate transpose) of the plan's transform, with the same
 * scale: adjoint(forward) = unnormalised inverse, adjoint(inverse) =
 * forward; for FFTGB_ORDER_BITREV plans the input is un-bit-reversed on load.
 */
int fftgb_exec_adjoint(fftgb_plan plan, const void *d_in, void *d_out,
                       int inverse, float scale, void *stream);

/*
 * Per-pass device timing.  While profiling is on, every fftgb_exec of this
 * plan (up to `max_execs` of them) records a CUDA event on its stream before
 * each kernel pass and after the last one; nothing synchronises.
 * fftgb_profile_end waits for those events and writes, for each pass index,
 * the summed milliseconds over the recorded executions.
 */
int fftgb_profile_begin(fftgb_plan plan, int max_execs);
int fftgb_profile_end(fftgb_plan plan, float *ms_per_pass, int npass,
                      int *nexec);
/* Kernel name of pass i, e.g. "k_cols<256>" (matches ncu launch lists). */
const char *fftgb_plan_pass_name(fftgb_plan plan, int i);

/*
 * Autotuner.  Times every decomposition the library has for the plan's
 * shape (per-axis passes, each fused two-pass tile shape, the single-pass
 * cluster kernel or the four-step for large 1D) on scratch buffers, keeps
 * the fastest in the plan, and records it in the tuning cache so later
 * plans of that shape start with it.  `report` (optional) receives the
 * timings, e.g. "axis=1.0430 fused:64:8=0.9895 ... -> fused:64:8".
 * The cache is a JSON object file: set with fftgb_tune_cache(), or the
 * FFTGB_TUNE_CACHE environment variable, or the `path` given to
 * fpga_initialize when that file is empty or already a JSON object.
 * fftgb_tune_cache(path) replaces the entries in memory with that file's;
 * NULL or "" forgets every entry (plans take the measured defaults) and
 * records nothing.
 */
int fftgb_plan_autotune(fftgb_plan plan, int reps, char *report,
                        size_t report_len);
int fftgb_tune_cache(const char *path);
/* The plan's decomposition: "axis", "axis:b8" (per-axis 3D with the
 * intermediate in the y-blocked layout [b][ny/8][nz][8][nx]: chosen where a
 * z-plane is 2 MiB or more; the plan owns a grid-sized work buffer and
 * fftgb_plan_inplace_ok() is 0), "fused:<rows>:<cols>[:p<mask>]"
 * (mask 16: pass A, 32: pass B as persistent kernels fed by TMA tensor
 * copies; 8: the one-tile passes with 8 points per thread, built for 64^3), "cluster[:<CTAs>]" (1D: one transform per thread-block cluster;
 * 3D: one grid of up to 2^18 points per 16-CTA cluster, one launch),
 * "fourstep", "mixed" (axes of lengths 2^a 3^b 5^c that are not powers of
 * two, one mixed-radix pass per axis; "mixed:simple": radix 16, 8, 4, 2, 5
 * and 3 stages only), "bluestein" (some axis of another length, or chosen:
 * Bluestein's algorithm) or "default" (single pass).  The autotuner times
 * the three non-power-of-two forms against each other. */
const char *fftgb_plan_variant(fftgb_plan plan);
/* FFTGB_ETIMEOUT if a bounded device-side wait of the plan's kernels gave up
 * since the last call (results invalid; synchronises and clears the flag):
 * the mbarrier waits of the TMA
 * tile copies (column passes, fused passes A and B), of the cluster 1D
 * kernel's bulk-copy exchange and of the tensor-core precision forms.
 * FFTGB_OK otherwise.  The fftfpga.h calls run this check after every
 * transform and return valid = false on a timeout.  No reference
 * counterpart. */
int fftgb_plan_status(fftgb_plan plan);

/* Test hook for the timeout path (no reference counterpart).  Runs the
 * give-up path of one family's bounded device wait: one thread waits on an
 * mbarrier that nothing arrives on, gives up after `polls` polls (at most
 * 2^20) and sets that family's status word, exactly as a kernel whose wait
 * gave up does; no copy is left in flight.  The next fftgb_plan_status of a
 * plan using that family (or the next fftfpga.h call on such a plan) then
 * reports the timeout and clears it.  Synchronises the device. */
#define FFTGB_WAIT_COLS_TMA 1    /* k_cols_tma tile copies */
#define FFTGB_WAIT_FUSED_TMA 2   /* k_xy_tma / k_rz_tma tile copies */
#define FFTGB_WAIT_CLUSTER_1D 3  /* k_1d_push bulk-copy exchange */
#define FFTGB_WAIT_TENSOR_CORE 4 /* tcgen05 MMA completion */
int fftgb_debug_expire_wait(int family, unsigned polls);

/* Spectral filters applied to a transform's outputs (no reference
 * counterpart).  FFTGB_FILTER_POISSON multiplies output (kx, ky, kz) by the
 * Poisson Green's function G = 1/|k|^2 (G = 0 at k = 0) on the integer
 * wavenumber grid k = n * fftfreq(n) per axis (index i < (n + 1)/2 is i,
 * else i - n).  The fused 3D plans apply it in the pass that stores the outputs;
 * other 3D plans add one element-wise pass.
 * fftgb_exec_filtered: filter(transform(in)) with transform as fftgb_exec.
 * fftgb_exec_adjoint_filtered: filter(adjoint(in)) (the adjoint of
 * "transform then filter" is "filter then adjoint"; since the filter is
 * real and diagonal, chaining the two calls builds the adjoint of a
 * filtered operator).  3D plans (any sides the plans take). */
#define FFTGB_FILTER_POISSON 1
int fftgb_exec_filtered(fftgb_plan plan, const void *d_in, void *d_out,
                        int inverse, float scale, int filter, void *stream);
int fftgb_exec_adjoint_filtered(fftgb_plan plan, const void *d_in, void *d_out,
                                int inverse, float scale, int filter,
                                void *stream);
/* r = a - b element-wise over n complex points (d_r may be NULL: not
 * stored) and *d_sum += sum |a - b|^2, accumulated in FP64 (the caller
 * zeroes *d_sum).  Device pointers, asynchronous on `stream`: the residual
 * and value of a least-squares loss in one pass. */
int fftgb_residual_sq(const void *d_a, const void *d_b, void *d_r, size_t n,
                      double *d_sum, void *stream);

/* Real-data transforms (no reference counterpart: the reference has complex
 * transforms only).  A plan of rank 1-3 over real grids [batch][nz][ny][nx]
 * (unused sizes 1; nx even, 4..8192, with nx/2 a power of two or
 * 2^a 3^b 5^c; ny and nz powers of two up to 4096 or 2^a 3^b 5^c up to 8192)
 * and their half spectra [batch][nz][ny][nx/2 + 1] complex, x fastest.
 * fftgb_exec_r2c: forward (sign -), real -> half spectrum.
 * fftgb_exec_c2r: backward (sign +), half spectrum -> real, unnormalised
 * (c2r(r2c(x)) = nx*ny*nz * x), the input is not modified.
 * Device pointers; out of place; `scale` multiplies the outputs. */
typedef struct fftgb_rplan_s *fftgb_rplan;
int fftgb_plan_r2c(fftgb_rplan *plan, int rank, unsigned nx, unsigned ny,
                   unsigned nz, unsigned batch);
void fftgb_rplan_destroy(fftgb_rplan plan);
size_t fftgb_rplan_real_points(fftgb_rplan plan);
size_t fftgb_rplan_spectrum_points(fftgb_rplan plan);
int fftgb_exec_r2c(fftgb_rplan plan, const float *d_real, void *d_spectrum,
                   float scale, void *stream);
int fftgb_exec_c2r(fftgb_rplan plan, const void *d_spectrum, float *d_real,
                   float scale, void *stream);

/* Ragged batch: `count` 3D grids of independent shapes, packed back to back
 * in the order given (grid g starts after grids 0..g-1).  Sides are powers of
 * two, or any lengths fftgb_plan_3d takes (2^a 3^b 5^c, others up to 2048):
 * those grids run as plans of their own inside the same graph. */
typedef struct {
  unsigned nx, ny, nz;
} fftgb_shape3;

typedef struct fftgb_ragged_s *fftgb_ragged;

int fftgb_ragged_plan(fftgb_ragged *plan, const fftgb_shape3 *shapes,
                      unsigned count, unsigned flags);
void fftgb_ragged_destroy(fftgb_ragged plan);
size_t fftgb_ragged_points(fftgb_ragged plan);
/* Runs the whole batch as one CUDA-graph launch.  When every axis length is
 * 16..512 the graph holds one persistent kernel that works through the
 * grids' tiles (axis by axis, each grid's next axis starting as soon as its
 * previous one is done), except for grids of 256 x 256 x {128, 256} (nz x
 * ny x nx): those run as grouped launches of the uniform plan's two
 * TMA-fed passes, up to 14 grids a launch (FFTGB_RAGGED_NO_GROUP=1 keeps
 * them in the persistent kernel); other shapes fall back to one plan per
 * grid inside the graph.  Input and output must not overlap. */
int fftgb_ragged_exec(fftgb_ragged plan, const void *d_in, void *d_out,
                      int inverse, void *stream);
/* Kernel launches per execution: 1 for the persistent kernel (when any grid
 * remains in it), 2 per grouped launch pair, plus the launches of the
 * per-grid plans. */
int fftgb_ragged_launches(fftgb_ragged plan);
/* FFTGB_ETIMEOUT if a dependency wait of the persistent kernel, a TMA
 * completion wait of the grouped passes or a bounded wait of a per-grid plan
 * gave up since the last call (synchronises), else FFTGB_OK. */
int fftgb_ragged_status(fftgb_ragged plan);
/* Test hook (no reference counterpart): runs the give-up path of the
 * persistent kernel's dependency wait once on this plan's status word (a
 * wait for a counter that never reaches its target, `polls` polls of about
 * 0.1 us, at most 2^20), so the next fftgb_ragged_status reports
 * FFTGB_ETIMEOUT.  FFTGB_EUNSUP for plans without a persistent kernel. */
int fftgb_ragged_debug_expire(fftgb_ragged plan, unsigned polls);

/*
 * fftgb_c2c_1d_noalloc - no counterpart in the reference.  The transform of
 * fftfpgaf_c2c_1d (N-point C2C, output bit-reversed within each block) on
 * caller-owned device buffers, for callers that cannot call cudaMalloc:
 * applications whose device memory is owned by their own pool allocator,
 * and hot paths that must not allocate because cudaMalloc can synchronise
 * the device.  It allocates nothing: its scratch is a file-scope device
 * array of FFTGB_NOALLOC_MAX_N points (8 MiB), held by every GPU that loads
 * the library until the process exits.
 *
 *   n        power of two, 2 <= n <= FFTGB_NOALLOC_MAX_N (larger n returns
 *            FFTGB_EUNSUP); any batch >= 1 (processed in rounds that fit
 *            the scratch)
 *   d_in     device pointer, n*batch float2, not modified
 *   d_out    device pointer, n*batch float2, must not overlap d_in
 *   stream   cudaStream_t (NULL: default stream)
 *
 * The first call on a device sets up that device (with the device current);
 * make it before any stream capture.  cudaDeviceReset after that first call
 * is not supported (the device's tables are not uploaded again).  Calls
 * share the scratch array: calls
 * that overlap on the GPU race.  fftgb_noalloc_last_error() explains a
 * non-zero status.
 */
#define FFTGB_NOALLOC_MAX_N (1u << 20)
int fftgb_c2c_1d_noalloc(unsigned n, unsigned batch, const void *d_in,
                         void *d_out, int inverse, void *stream);
const char *fftgb_noalloc_last_error(void);

/* Checks the tensor-core (tcgen05) path on the current GPU: a 128x32x32
 * half-precision (bf16 != 0: bfloat16) product with FP32 accumulation
 * against an FP64 product on the host; *max_rel_err receives the largest
 * error relative to the largest output. */
int fftgb_tc_selftest(int bf16, float *max_rel_err);

/* Text of the last error on the calling thread ("" if none). */
const char *fftgb_last_error(void);

/* Library version string. */
const char *fftgb_version(void);

#ifdef __cplusplus
}
#endif

#endif /* FFTFPGA_EXT_H */
