/*
 * fft1d.c - 1D entry points of the C host library.  Mirrors the reference's
 * api/src/fft1d.c: argument validation returns an fpga_t with valid == false
 * before any device work, then the transform runs through the CUDA shim.
 * Output is bit-reversed within each N-point block, as the reference's
 * engine stores it (kernels/common/fft_8.cl:28-30).
 */
#include <stdbool.h>
#include <stdlib.h>
#include <string.h>

#include "fftfpga.h"
#include "fftfpga_ext.h"
#include "../../shim/shim.h"

static fpga_t invalid_result(void) {
  fpga_t t;
  memset(&t, 0, sizeof(t));
  return t;
}

static bool pow2(unsigned n) { return (n & (n - 1)) == 0; }

/*
 * Reference api/src/fft1d.c:27-137.  The reference has no double-precision
 * kernel and reads back sizeof(float2) per point (fft1d.c:113); here the
 * input is rounded to float2, the FP32 path runs, and the result is widened.
 */
fpga_t fftfpga_c2c_1d(const unsigned N, const double2 *inp, double2 *out,
                      const bool inv, const unsigned iter) {
  if (inp == NULL || out == NULL || !pow2(N) || N == 0 || iter == 0)
    return invalid_result();
  const size_t n = (size_t)N * iter;
  float2 *a = (float2 *)malloc(n * sizeof(float2));
  float2 *b = (float2 *)malloc(n * sizeof(float2));
  if (a == NULL || b == NULL) {
    free(a);
    free(b);
    return invalid_result();
  }
  for (size_t i = 0; i < n; i++) {
    a[i].x = (float)inp[i].x;
    a[i].y = (float)inp[i].y;
  }
  fpga_t t = fftgb_shim_run(N, 1, 1, iter, FFTGB_ORDER_BITREV, a, b, inv,
                            FFTGB_RUN_COPY);
  if (t.valid) {
    for (size_t i = 0; i < n; i++) {
      out[i].x = (double)b[i].x;
      out[i].y = (double)b[i].y;
    }
  }
  free(a);
  free(b);
  return t;
}

/* Reference api/src/fft1d.c:148-247. */
fpga_t fftfpgaf_c2c_1d(const unsigned N, const float2 *inp, float2 *out,
                       const bool inv, const unsigned iter) {
  if (inp == NULL || out == NULL || !pow2(N) || N == 0 || iter == 0)
    return invalid_result();
  return fftgb_shim_run(N, 1, 1, iter, FFTGB_ORDER_BITREV, inp, out, inv,
                        FFTGB_RUN_COPY);
}

/* Reference api/src/fft1d.c:258-373: invalid unless initialised with SVM. */
fpga_t fftfpgaf_c2c_1d_svm(const unsigned N, const float2 *inp, float2 *out,
                           const bool inv, const unsigned batch) {
  if (inp == NULL || out == NULL || !pow2(N) || N == 0 || batch == 0 ||
      !fftgb_shim_svm_enabled())
    return invalid_result();
  return fftgb_shim_run(N, 1, 1, batch, FFTGB_ORDER_BITREV, inp, out, inv,
                        FFTGB_RUN_SVM);
}
