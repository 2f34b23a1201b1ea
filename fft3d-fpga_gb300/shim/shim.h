/*
 * shim.h - internal C interface between the C host library (api/src) and
 * the C++/CUDA shim.  Not installed; callers use fftfpga.h / fftfpga_ext.h.
 *
 * The shim replaces the reference's OpenCL plumbing (api/src/fftfpga.c:18-29
 * globals, queue_setup/queue_cleanup :147-188, opencl_utils.c, svm.c): it
 * owns the CUDA device, a stream, cached device buffers, device-mapped host
 * staging buffers, twiddle tables and a plan cache.  It never calls exit().
 */
#ifndef FFTGB_SHIM_H
#define FFTGB_SHIM_H

#include <stdbool.h>

#include "fftfpga.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Return codes as fpga_initialize (0, -1 .. -5). */
int fftgb_shim_initialize(const char *platform_name, const char *path,
                          bool use_svm);
void fftgb_shim_final(void);
/* 1 once fpga_initialize succeeded with use_svm. */
int fftgb_shim_svm_enabled(void);

/* How a host-buffer transform moves data. */
#define FFTGB_RUN_COPY 0     /* H2D copy, kernels, D2H copy; times each
                                (batches above 64 MiB in overlapped chunks,
                                the times then summed over the chunks)      */
#define FFTGB_RUN_PIPELINE 1 /* per-grid copies overlapped with compute;
                                exec_t = wall time of the whole call        */
#define FFTGB_RUN_SVM 2      /* through device-mapped host staging          */

/*
 * Run `batch` transforms of a grid with dims (nx, ny, nz) on host buffers
 * (unused trailing dims are 1).  flags: FFTGB_ORDER_* of fftfpga_ext.h.
 * Arguments must already be validated by the caller.
 */
fpga_t fftgb_shim_run(unsigned nx, unsigned ny, unsigned nz, unsigned batch,
                      unsigned flags, const float2 *inp, float2 *out,
                      bool inv, int mode);

#ifdef __cplusplus
}
#endif

#endif
