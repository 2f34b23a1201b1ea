/*
 * fftfpga.c - device set-up, release and host allocation of the C host
 * library.  Mirrors the reference's api/src/fftfpga.c (same entry points,
 * same return codes); the OpenCL platform/context/program handling of the
 * reference (fftfpga.c:72-130) is replaced by the CUDA shim.
 */
#define _POSIX_C_SOURCE 200112L
#include <stdbool.h>
#include <stdlib.h>

#include "fftfpga.h"
#include "../../shim/shim.h"

/* 64-byte aligned allocation, as alignedMalloc (api/src/opencl_utils.c:
 * 205-213).  The caller releases it with free(). */
static void *aligned_alloc64(size_t sz) {
  void *p = NULL;
  if (posix_memalign(&p, 64, sz) != 0) return NULL;
  return p;
}

/* Reference api/src/fftfpga.c:37-44: NULL for size 0. */
void *fftfpga_complex_malloc(const size_t sz) {
  if (sz == 0) return NULL;
  return aligned_alloc64(sz);
}

/* Reference api/src/fftfpga.c:52-58: NULL for size 0. */
void *fftfpgaf_complex_malloc(const size_t sz) {
  if (sz == 0) return NULL;
  return aligned_alloc64(sz);
}

/* Reference api/src/fftfpga.c:72-130.  Codes: 0 ok, -1 no path, -2 no
 * matching platform, -3 no device, -4 path unreadable, -5 no SVM. */
int fpga_initialize(const char *platform_name, const char *path,
                    const bool use_svm) {
  return fftgb_shim_initialize(platform_name, path, use_svm);
}

/* Reference api/src/fftfpga.c:135-142. */
void fpga_final(void) { fftgb_shim_final(); }
