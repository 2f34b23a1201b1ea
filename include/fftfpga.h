/*
 * fftfpga.h - drop-in C ABI of FFTFPGA's public API, served by GB300 kernels.
 *
 * Every declaration below keeps the exact name, signature and struct layout
 * of the reference header api/include/fftfpga/fftfpga.h, so existing callers
 * (the reference's examples/fft.cpp, its gtest suite, CP2K) relink against
 * libfftfpga.so unchanged.  Each entry point cites the declaration it
 * replaces.  Semantics kept from the reference:
 *
 *   - out-of-place, synchronous; `inp` is never modified; both are HOST
 *     pointers;
 *   - forward sign -, inverse unnormalised (no 1/N);
 *   - 1D output bit-reversed within each N-point block, 2D/3D natural order;
 *   - invalid arguments (NULL pointer, N not a power of two, bad batch)
 *     return an fpga_t with valid == false and touch no memory.
 *
 * Deliberate deviations (documented, not silent):
 *   - a runtime failure returns valid == false instead of calling exit();
 *   - N is a runtime value (any power of two that fits), not fixed by a
 *     bitstream; `interleaving` (a DDR bank hint) is accepted and ignored;
 *   - fftfpgaf_c2c_2d_bram honours how_many > 1.
 */
#ifndef FFTFPGA_H
#define FFTFPGA_H

#include <stdbool.h>
#include <stddef.h>

#if defined(__CUDACC__) || defined(__VECTOR_TYPES_H__)
/* CUDA translation units already define float2/double2 with the same members
 * in the same order (x = real, y = imaginary) and the same size. */
#include <vector_types.h>
#else
/* Single precision complex, {re, im}.  Reference fftfpga.h:16-19. */
typedef struct {
  float x; /* real */
  float y; /* imaginary */
} float2;

/* Double precision complex, {re, im}.  Reference fftfpga.h:24-27. */
typedef struct {
  double x; /* real */
  double y; /* imaginary */
} double2;
#endif

/*
 * Per-call timing in milliseconds.  Reference fftfpga.h:32-39.
 *   pcie_write_t  host->device copy of the input (CUDA events)
 *   pcie_read_t   device->host copy of the output (CUDA events)
 *   exec_t        device kernel time of the transform (CUDA events); for
 *                 fftfpgaf_c2c_3d_ddr_batch the whole pipelined call, copies
 *                 included, as in the reference (api/src/fft3d.c:489,861)
 *   svm_copyin_t  host copy into the device-mapped staging buffer
 *   svm_copyout_t host copy out of the device-mapped staging buffer
 *   valid         true when the transform ran and its output is written
 */
typedef struct fpga_timing {
  double pcie_read_t;
  double pcie_write_t;
  double exec_t;
  double svm_copyin_t;
  double svm_copyout_t;
  bool valid;
} fpga_t;

#ifdef __cplusplus
extern "C" {
#endif

/*
 * Select and set up the CUDA device.  Reference fftfpga.h:56
 * (api/src/fftfpga.c:72-130).  Return codes keep the reference meaning:
 *    0  success
 *   -1  `path` NULL or empty
 *   -2  `platform_name` NULL/empty or matches (case-insensitive substring)
 *       neither "NVIDIA CUDA" nor the device name
 *   -3  no CUDA device
 *   -4  `path` names no readable file (kept as the plan-cache file)
 *   -5  use_svm requested but the device cannot read host memory directly
 */
int fpga_initialize(const char *platform_name, const char *path,
                    const bool use_svm);

/* Release every device resource the library holds.  Reference fftfpga.h:61. */
void fpga_final(void);

/* 64-byte aligned host allocation, NULL for size 0; release with free().
 * Reference fftfpga.h:68 and :75 (api/src/fftfpga.c:37-58). */
void *fftfpga_complex_malloc(const size_t sz);
void *fftfpgaf_complex_malloc(const size_t sz);

/* Double precision 1D: converted to float2, run on the FP32 path, converted
 * back.  Reference fftfpga.h:86 (whose implementation reads back only
 * sizeof(float2) per point, api/src/fft1d.c:113). */
fpga_t fftfpga_c2c_1d(const unsigned N, const double2 *inp, double2 *out,
                      const bool inv, const unsigned iter);

/* `iter` N-point 1D FFTs, output bit-reversed per block.
 * Reference fftfpga.h:97 (api/src/fft1d.c:148-247). */
fpga_t fftfpgaf_c2c_1d(const unsigned N, const float2 *inp, float2 *out,
                       const bool inv, const unsigned iter);

/* Same through device-mapped host staging; needs fpga_initialize(.., true).
 * Reference fftfpga.h:108 (api/src/fft1d.c:258-373). */
fpga_t fftfpgaf_c2c_1d_svm(const unsigned N, const float2 *inp, float2 *out,
                           const bool inv, const unsigned batch);

/* `how_many` N x N 2D FFTs.  Reference fftfpga.h:120 (api/src/fft2d.c:170-338). */
fpga_t fftfpgaf_c2c_2d_bram(const unsigned N, const float2 *inp, float2 *out,
                            const bool inv, const bool interleaving,
                            const unsigned how_many);

/* Reference fftfpga.h:131 (api/src/fft2d.c:348-505). */
fpga_t fftfpgaf_c2c_2d_bram_svm(const unsigned N, const float2 *inp,
                                float2 *out, const bool inv,
                                const unsigned how_many);

/* One N x N 2D FFT.  Reference fftfpga.h:141 (api/src/fft2d.c:27-159). */
fpga_t fftfpgaf_c2c_2d_ddr(const unsigned N, const float2 *inp, float2 *out,
                           const bool inv);

/* One N^3 3D FFT, on-chip variant.  Reference fftfpga.h:152
 * (api/src/fft3d.c:30-196). */
fpga_t fftfpgaf_c2c_3d_bram(const unsigned N, const float2 *inp, float2 *out,
                            const bool inv, const bool interleaving);

/* One N^3 3D FFT.  Reference fftfpga.h:162 (api/src/fft3d.c:206-384). */
fpga_t fftfpgaf_c2c_3d_ddr(const unsigned N, const float2 *inp, float2 *out,
                           const bool inv);

/* `how_many` >= 2 N^3 3D FFTs, copies overlapped with compute.
 * Reference fftfpga.h:164 (api/src/fft3d.c:396-913). */
fpga_t fftfpgaf_c2c_3d_ddr_batch(const unsigned N, const float2 *inp,
                                 float2 *out, const bool inv,
                                 const bool interleaving,
                                 const unsigned how_many);

/* Reference fftfpga.h:175 (api/src/fft3d_svm.c:31-232). */
fpga_t fftfpgaf_c2c_3d_ddr_svm(const unsigned N, const float2 *inp,
                               float2 *out, const bool inv,
                               const bool interleaving);

/* `how_many` >= 1 grids.  Reference fftfpga.h:186 (api/src/fft3d_svm.c:244-520). */
fpga_t fftfpgaf_c2c_3d_ddr_svm_batch(const unsigned N, const float2 *inp,
                                     float2 *out, const bool inv,
                                     const unsigned how_many);

#ifdef __cplusplus
}
#endif

#endif /* FFTFPGA_H */
