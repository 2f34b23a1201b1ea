/*
 * fft2d.c - 2D entry points of the C host library.  Mirrors the reference's
 * api/src/fft2d.c.  Both the _ddr and _bram variants compute the same
 * natural-order N x N transform; on the GPU the row pass and the strided
 * column pass replace the reference's fetch/fft/transpose rounds
 * (fft2d.c:77-114) and its on-chip transpose pipeline (fft2d.c:170-338).
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

/* Reference api/src/fft2d.c:27-159: one N x N transform. */
fpga_t fftfpgaf_c2c_2d_ddr(const unsigned N, const float2 *inp, float2 *out,
                           const bool inv) {
  if (inp == NULL || out == NULL || !pow2(N)) return invalid_result();
  return fftgb_shim_run(N, N, 1, 1, 0, inp, out, inv, FFTGB_RUN_COPY);
}

/* Reference api/src/fft2d.c:170-338.  `interleaving` is a DDR bank hint and
 * is ignored; how_many > 1 is honoured (the reference kernel runs its second
 * stage once, kernels/fft2d/fft2d_bram.cl:190). */
fpga_t fftfpgaf_c2c_2d_bram(const unsigned N, const float2 *inp, float2 *out,
                            const bool inv, const bool interleaving,
                            const unsigned how_many) {
  (void)interleaving;
  if (inp == NULL || out == NULL || !pow2(N) || how_many == 0)
    return invalid_result();
  return fftgb_shim_run(N, N, 1, how_many, 0, inp, out, inv, FFTGB_RUN_COPY);
}

/* Reference api/src/fft2d.c:348-505: invalid unless initialised with SVM. */
fpga_t fftfpgaf_c2c_2d_bram_svm(const unsigned N, const float2 *inp,
                                float2 *out, const bool inv,
                                const unsigned how_many) {
  if (inp == NULL || out == NULL || !pow2(N) || how_many == 0 ||
      !fftgb_shim_svm_enabled())
    return invalid_result();
  return fftgb_shim_run(N, N, 1, how_many, 0, inp, out, inv, FFTGB_RUN_SVM);
}
