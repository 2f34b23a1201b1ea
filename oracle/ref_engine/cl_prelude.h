/*
 * Test infrastructure only (oracle). Never linked into the product library.
 *
 * Minimal OpenCL-C vocabulary so that the reference's FFT engine source
 * (kernels/common/fft_8.cl, which includes kernels/common/twid_radix4_8.cl)
 * compiles unchanged as C++ on the host.  The engine is used only to produce
 * golden 1D vectors that pin the output order, sign and inverse convention
 * of fftfpgaf_c2c_1d.
 *
 * What OpenCL provides and C++ lacks:
 *   - the float2 vector type with component-wise + and -   (fft_8.cl:61-72)
 *   - the `constant` address-space qualifier                (twid_radix4_8.cl:27)
 *   - M_PI_F, the float value of pi                          (fft_8.cl:224)
 *   - float overloads of cos/sin                             (fft_8.cl:240-241)
 */
#ifndef FFTGB_ORACLE_CL_PRELUDE_H
#define FFTGB_ORACLE_CL_PRELUDE_H

#include <math.h>

struct float2 {
  float x;
  float y;
};

static inline float2 operator+(float2 a, float2 b) {
  float2 r;
  r.x = a.x + b.x;
  r.y = a.y + b.y;
  return r;
}

static inline float2 operator-(float2 a, float2 b) {
  float2 r;
  r.x = a.x - b.x;
  r.y = a.y - b.y;
  return r;
}

#define constant const
#define M_PI_F ((float)M_PI)

#endif
