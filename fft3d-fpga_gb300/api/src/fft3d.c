/*
 * fft3d.c - 3D entry points of the C host library.  Mirrors the reference's
 * api/src/fft3d.c and api/src/fft3d_svm.c: same validation rules, same
 * natural-order output, same fpga_t meaning.  The reference's 7-kernel
 * channel pipeline with its DDR transpose (fft3d.c:206-384) becomes the
 * shim's pass plan; the _bram variant (on-chip transpose, fft3d.c:30-196)
 * computes the identical transform.
 */
#include <stdbool.h>
#include <stddef.h>
#include <string.h>

#include "fftfpga.h"
#include "fftfpga_ext.h"
#include "../../shim/shim.h"

static fpga_t invalid_result(void) {
  fpga_t t;
  memset(&t, 0, sizeof(t));
  return t;
}

static bool pow2(unsigned n) { return n != 0 && (n & (n - 1)) == 0; }

/* Reference api/src/fft3d.c:30-196. */
fpga_t fftfpgaf_c2c_3d_bram(const unsigned N, const float2 *inp, float2 *out,
                            const bool inv, const bool interleaving) {
  (void)interleaving;
  if (inp == NULL || out == NULL || !pow2(N)) return invalid_result();
  return fftgb_shim_run(N, N, N, 1, 0, inp, out, inv, FFTGB_RUN_COPY);
}

/* Reference api/src/fft3d.c:206-384. */
fpga_t fftfpgaf_c2c_3d_ddr(const unsigned N, const float2 *inp, float2 *out,
                           const bool inv) {
  if (inp == NULL || out == NULL || !pow2(N)) return invalid_result();
  return fftgb_shim_run(N, N, N, 1, 0, inp, out, inv, FFTGB_RUN_COPY);
}

/* Reference api/src/fft3d.c:396-913: how_many >= 2 (fft3d.c:403); grid i at
 * inp[i*N^3]; exec_t is the wall time of the whole call, transfers included
 * (fft3d.c:489, 861), pcie_* stay 0. */
fpga_t fftfpgaf_c2c_3d_ddr_batch(const unsigned N, const float2 *inp,
                                 float2 *out, const bool inv,
                                 const bool interleaving,
                                 const unsigned how_many) {
  (void)interleaving;
  if (inp == NULL || out == NULL || !pow2(N) || how_many <= 1)
    return invalid_result();
  return fftgb_shim_run(N, N, N, how_many, 0, inp, out, inv,
                        FFTGB_RUN_PIPELINE);
}

/* Reference api/src/fft3d_svm.c:31-232: invalid unless initialised with
 * SVM (fft3d_svm.c:40). */
fpga_t fftfpgaf_c2c_3d_ddr_svm(const unsigned N, const float2 *inp,
                               float2 *out, const bool inv,
                               const bool interleaving) {
  (void)interleaving;
  if (inp == NULL || out == NULL || !pow2(N) || !fftgb_shim_svm_enabled())
    return invalid_result();
  return fftgb_shim_run(N, N, N, 1, 0, inp, out, inv, FFTGB_RUN_SVM);
}

/* Reference api/src/fft3d_svm.c:244-520: how_many >= 1 (fft3d_svm.c:251). */
fpga_t fftfpgaf_c2c_3d_ddr_svm_batch(const unsigned N, const float2 *inp,
                                     float2 *out, const bool inv,
                                     const unsigned how_many) {
  if (inp == NULL || out == NULL || !pow2(N) || how_many == 0 ||
      !fftgb_shim_svm_enabled())
    return invalid_result();
  return fftgb_shim_run(N, N, N, how_many, 0, inp, out, inv, FFTGB_RUN_SVM);
}
