/*
 * Replays the assertions of the reference's gtest suite against
 * libfftfpga.so, from C, through include/fftfpga.h:
 *   tests/test_fft1d_fpga.cpp:16-70, tests/test_fft2d_fpga.cpp:17-62,
 *   tests/test_fft3d_fpga.cpp:16-94, tests/test_fft_setup.cpp:16-47.
 *
 *   test_validity            checks that need no GPU (init codes -1, -2, and
 *                            -3 when no device is present)
 *   test_validity gpu FILE   also the codes that need the device: -4, 0 with
 *                            the readable FILE, SVM checks after init
 * Exit status 0 when every check passes.
 */
#include <stdio.h>
#include <stdlib.h>

#include "fftfpga.h"

static int failures = 0;

#define EXPECT_EQ(a, b)                                                   \
  do {                                                                    \
    long long a_ = (long long)(a), b_ = (long long)(b);                   \
    if (a_ != b_) {                                                       \
      fprintf(stderr, "%s:%d: %s == %lld, expected %lld\n", __FILE__,     \
              __LINE__, #a, a_, b_);                                      \
      failures++;                                                         \
    }                                                                     \
  } while (0)

static void fft1d_validity(void) {
  const unsigned N = 1u << 6;
  float2 *test = (float2 *)malloc(sizeof(float2) * N);
  fpga_t t;
  t = fftfpgaf_c2c_1d(N, NULL, test, false, 1);
  EXPECT_EQ(t.valid, 0);
  t = fftfpgaf_c2c_1d(N, test, NULL, false, 1);
  EXPECT_EQ(t.valid, 0);
  t = fftfpgaf_c2c_1d(N - 1, test, test, false, 1);
  EXPECT_EQ(t.valid, 0);
  /* svm not enabled */
  t = fftfpgaf_c2c_1d_svm(N, test, test, false, 1);
  EXPECT_EQ(t.valid, 0);
  free(test);
}

static void fft2d_validity(void) {
  const unsigned N = 64;
  float2 *test = (float2 *)malloc(sizeof(float2) * N * N);
  fpga_t t;
  t = fftfpgaf_c2c_2d_bram(64, NULL, test, 0, 0, 1);
  EXPECT_EQ(t.valid, 0);
  t = fftfpgaf_c2c_2d_bram(64, test, NULL, 0, 0, 1);
  EXPECT_EQ(t.valid, 0);
  t = fftfpgaf_c2c_2d_bram(63, test, test, 0, 0, 1);
  EXPECT_EQ(t.valid, 0);
  t = fftfpgaf_c2c_2d_ddr(64, NULL, test, 0);
  EXPECT_EQ(t.valid, 0);
  t = fftfpgaf_c2c_2d_ddr(64, test, NULL, 0);
  EXPECT_EQ(t.valid, 0);
  t = fftfpgaf_c2c_2d_ddr(63, test, test, 0);
  EXPECT_EQ(t.valid, 0);
  free(test);
}

static void fft3d_validity(void) {
  const unsigned N = 64;
  float2 *test = (float2 *)malloc(sizeof(float2) * N * N * N * 2);
  fpga_t t;
  t = fftfpgaf_c2c_3d_bram(64, NULL, test, 0, 0);
  EXPECT_EQ(t.valid, 0);
  t = fftfpgaf_c2c_3d_bram(64, test, NULL, 0, 0);
  EXPECT_EQ(t.valid, 0);
  t = fftfpgaf_c2c_3d_bram(63, test, test, 0, 0);
  EXPECT_EQ(t.valid, 0);
  t = fftfpgaf_c2c_3d_ddr(64, NULL, test, 0);
  EXPECT_EQ(t.valid, 0);
  t = fftfpgaf_c2c_3d_ddr(64, test, NULL, 0);
  EXPECT_EQ(t.valid, 0);
  t = fftfpgaf_c2c_3d_ddr(63, test, test, 0);
  EXPECT_EQ(t.valid, 0);
  t = fftfpgaf_c2c_3d_ddr_svm_batch(64, NULL, test, 0, 2);
  EXPECT_EQ(t.valid, 0);
  t = fftfpgaf_c2c_3d_ddr_svm_batch(64, test, NULL, 0, 2);
  EXPECT_EQ(t.valid, 0);
  t = fftfpgaf_c2c_3d_ddr_svm_batch(63, test, test, 0, 2);
  EXPECT_EQ(t.valid, 0);
  t = fftfpgaf_c2c_3d_ddr_svm_batch(63, test, test, 0, 0);
  EXPECT_EQ(t.valid, 0);
  t = fftfpgaf_c2c_3d_ddr_svm_batch(63, test, test, 0, (unsigned)-1);
  EXPECT_EQ(t.valid, 0);
  /* batch variant needs how_many >= 2 (api/src/fft3d.c:403) */
  t = fftfpgaf_c2c_3d_ddr_batch(64, test, test, 0, 0, 1);
  EXPECT_EQ(t.valid, 0);
  t = fftfpgaf_c2c_3d_ddr_batch(64, test, test, 0, 0, 0);
  EXPECT_EQ(t.valid, 0);
  free(test);
}

static void setup_codes(int gpu, const char *file) {
  EXPECT_EQ(fpga_initialize("NVIDIA CUDA", "", false), -1);
  EXPECT_EQ(fpga_initialize("NVIDIA CUDA", NULL, false), -1);
  EXPECT_EQ(fpga_initialize("TEST", "fft1d_emulate.aocx", false), -2);
  EXPECT_EQ(fpga_initialize("", "x", false), -2);
  if (!gpu) {
    EXPECT_EQ(fpga_initialize("NVIDIA CUDA", "x", false), -3);
    EXPECT_EQ(fpga_initialize("nvidia", "x", true), -3);
  } else {
    EXPECT_EQ(fpga_initialize("NVIDIA CUDA", "TEST", false), -4);
    EXPECT_EQ(fpga_initialize("nvidia", file, false), 0);
    fpga_final();
  }
  EXPECT_EQ(fftfpga_complex_malloc(0) == NULL, 1);
  EXPECT_EQ(fftfpgaf_complex_malloc(0) == NULL, 1);
  void *p = fftfpgaf_complex_malloc(1000);
  EXPECT_EQ(p != NULL, 1);
  EXPECT_EQ(((unsigned long)p) % 64, 0);
  free(p);
}

static void svm_after_init(const char *file) {
  const unsigned N = 64;
  float2 *test = (float2 *)calloc(N, sizeof(float2));
  EXPECT_EQ(fpga_initialize("NVIDIA CUDA", file, true), 0);
  fpga_t t = fftfpgaf_c2c_1d_svm(N, NULL, test, false, 1);
  EXPECT_EQ(t.valid, 0);
  t = fftfpgaf_c2c_1d_svm(N, test, NULL, false, 1);
  EXPECT_EQ(t.valid, 0);
  t = fftfpgaf_c2c_1d_svm(N - 1, test, test, false, 1);
  EXPECT_EQ(t.valid, 0);
  float2 *out = (float2 *)calloc(N, sizeof(float2));
  test[0].x = 1.0f;
  t = fftfpgaf_c2c_1d_svm(N, test, out, false, 1);
  EXPECT_EQ(t.valid, 1);
  /* FFT of a delta is all ones, in any order */
  for (unsigned i = 0; i < N; i++) {
    EXPECT_EQ(out[i].x > 0.9999f && out[i].x < 1.0001f, 1);
  }
  fpga_final();
  free(test);
  free(out);
}

int main(int argc, char **argv) {
  const int gpu = argc > 2;
  fft1d_validity();
  fft2d_validity();
  fft3d_validity();
  setup_codes(gpu, gpu ? argv[2] : NULL);
  if (gpu) svm_after_init(argv[2]);
  EXPECT_EQ(sizeof(fpga_t), 48);
  EXPECT_EQ(sizeof(float2), 8);
  EXPECT_EQ(sizeof(double2), 16);
  printf("%s: %d failure(s)\n", argv[0], failures);
  return failures ? 1 : 0;
}
