/*
 * Test infrastructure only (oracle). Never linked into the product library.
 *
 * Host driver around the reference's own radix-2^2 feed-forward FFT engine.
 * The engine arithmetic is NOT restated here: the reference source file
 * kernels/common/fft_8.cl is compiled in place (see Makefile in this folder)
 * and its `fft_step` is called exactly as the reference's fft1d task calls it.
 *
 * What this file restates (the data movement around the engine):
 *
 *  - fetch (kernels/fft1d/fft1d.cl:120-171).  For 64 <= N <= 4096 the
 *    reference builds use LOG_CONT_FACTOR = LOGN - 6, which makes
 *    permute_gid() (fft1d.cl:120-137) the identity and the work-group size
 *    N/8 (api/src/fft1d.c:200-201).  Work-item `lid` of group `t` loads
 *    points t*N + 8*lid .. +7 into local memory, and channel k then receives,
 *    in work-item order, buf[bit_reversed(k,3) * N/8 + lid].  So on engine
 *    step s of transform t, stream k carries x[t*N + bitrev3(k)*N/8 + s].
 *
 *  - the fft1d task loop (fft1d.cl:183-252): count*N/8 + N/8 - 1 steps, zero
 *    input once the inputs are exhausted, step index i % (N/8), and
 *    outputs written sequentially from step N/8 - 1 on, 8 points per step.
 *    The stored order is bit-reversed within each N-point block
 *    (fft_8.cl:28-30; examples/helper.cpp:143-162 undoes it).
 *
 * The engine's private delay line (fft1d.cl:192) is uninitialised in the
 * reference; it is zeroed here, which only affects outputs the task never
 * stores.
 */
#include "cl_prelude.h"

#include <stdlib.h>
#include <string.h>

#include "fft_8.cl"

static unsigned bitrev3(unsigned k) {
  return ((k & 1u) << 2) | (k & 2u) | ((k >> 2) & 1u);
}

extern "C" int ref_engine_fft1d(int logN, const float *in, float *out,
                                int count, int inverse) {
  if (logN < 3 || logN > 12 || count < 1 || in == NULL || out == NULL) {
    return -1;
  }
  const int N = 1 << logN;
  const int steps_per = N / 8;
  const int delay_len = N + 8 * (logN - 2);
  float2 *delay_line = (float2 *)calloc((size_t)delay_len, sizeof(float2));
  if (delay_line == NULL) {
    return -2;
  }
  const float2 *x = (const float2 *)in;
  float2 *y = (float2 *)out;
  const long total_steps = (long)count * steps_per + steps_per - 1;
  for (long i = 0; i < total_steps; i++) {
    float2x8 data;
    if (i < (long)count * steps_per) {
      const long t = i / steps_per;
      const long s = i % steps_per;
      const float2 *blk = x + t * N;
      data.i0 = blk[bitrev3(0) * steps_per + s];
      data.i1 = blk[bitrev3(1) * steps_per + s];
      data.i2 = blk[bitrev3(2) * steps_per + s];
      data.i3 = blk[bitrev3(3) * steps_per + s];
      data.i4 = blk[bitrev3(4) * steps_per + s];
      data.i5 = blk[bitrev3(5) * steps_per + s];
      data.i6 = blk[bitrev3(6) * steps_per + s];
      data.i7 = blk[bitrev3(7) * steps_per + s];
    } else {
      float2 z;
      z.x = 0.0f;
      z.y = 0.0f;
      data.i0 = data.i1 = data.i2 = data.i3 = z;
      data.i4 = data.i5 = data.i6 = data.i7 = z;
    }
    data = fft_step(data, (int)(i % steps_per), delay_line, inverse != 0, logN);
    if (i >= steps_per - 1) {
      float2 *dst = y + 8 * (i - (steps_per - 1));
      dst[0] = data.i0;
      dst[1] = data.i1;
      dst[2] = data.i2;
      dst[3] = data.i3;
      dst[4] = data.i4;
      dst[5] = data.i5;
      dst[6] = data.i6;
      dst[7] = data.i7;
    }
  }
  free(delay_line);
  return 0;
}
