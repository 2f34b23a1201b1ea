/* fft - command-line driver of libfftfpga.so with the options of the
 * reference's example program (examples/fft.cpp:8-101, options in
 * examples/helper.cpp:44-57):
 *
 *   fft -p <file> [-n N] [-d 1|2|3] [-b] [-i iter] [-c batch] [-y] [-t] [-m] [-s] [-e]
 *
 * It calls the same entry point the reference example selects for each
 * option combination, verifies every iteration against its own FP64 host
 * FFT (the reference verifies with FFTW single precision, absent here) by
 * the reference's rule, SNR > 120 dB (examples/helper.cpp:164-198), with
 * 1D outputs read in the bit-reversed order the 1D entry points store, and
 * prints the reference's measurement report (examples/helper.cpp:208-259)
 * with rates in real units: GB/s = 1e9 B/s and GFLOP/s = 1e9 flop/s (the
 * reference divides by 2^20 and 2^30).
 */
#define _POSIX_C_SOURCE 200809L
#include <getopt.h>
#include <math.h>
#include <stdbool.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fftfpga.h"

typedef struct {
  unsigned num, dim, iter, batch;
  bool inv, noverify, burst, use_bram, use_usm, emulate;
  const char *path;
} config_t;

static void usage(FILE *f) {
  fprintf(f,
          "Offloading FFT to the GPU (FFTFPGA C API)\n"
          "Usage: fft -p <path> [options]\n"
          "  -n, --num N        Number of sample points in a dimension (default 64)\n"
          "  -d, --dim D        Number of dimensions, 1-3 (default 3)\n"
          "  -b, --back         Toggle backward FFT\n"
          "  -i, --iter K       Number of iterations (default 1)\n"
          "  -p, --path FILE    Path given to fpga_initialize (plan-tuning cache)\n"
          "  -y, --noverify     Toggle to not verify against the FP64 host FFT\n"
          "  -c, --batch B      Number of batched transforms (default 1)\n"
          "  -t, --burst        Toggle burst interleaving (accepted, no effect on GPU)\n"
          "  -m, --use_bram     Toggle the _bram entry points\n"
          "  -s, --use_usm      Toggle the shared-virtual-memory entry points\n"
          "  -e, --emulate      Toggle emulation (not applicable: always the GPU)\n"
          "  -h, --help         Print usage\n");
}

static int parse_unsigned(const char *s, unsigned *v) {
  char *end = NULL;
  const unsigned long x = strtoul(s, &end, 10);
  if (!s[0] || *end || x > 0xffffffffUL) return -1;
  *v = (unsigned)x;
  return 0;
}

static int parse_args(int argc, char **argv, config_t *c) {
  static const struct option opts[] = {
      {"num", required_argument, 0, 'n'},   {"dim", required_argument, 0, 'd'},
      {"back", no_argument, 0, 'b'},        {"iter", required_argument, 0, 'i'},
      {"path", required_argument, 0, 'p'},  {"noverify", no_argument, 0, 'y'},
      {"batch", required_argument, 0, 'c'}, {"burst", no_argument, 0, 't'},
      {"use_bram", no_argument, 0, 'm'},    {"use_usm", no_argument, 0, 's'},
      {"emulate", no_argument, 0, 'e'},     {"help", no_argument, 0, 'h'},
      {0, 0, 0, 0}};
  memset(c, 0, sizeof(*c));
  c->num = 64;
  c->dim = 3;
  c->iter = 1;
  c->batch = 1;
  int o;
  while ((o = getopt_long(argc, argv, "n:d:bi:p:yc:tmseh", opts, NULL)) != -1) {
    switch (o) {
      case 'n': if (parse_unsigned(optarg, &c->num)) return 1; break;
      case 'd': if (parse_unsigned(optarg, &c->dim)) return 1; break;
      case 'b': c->inv = true; break;
      case 'i': if (parse_unsigned(optarg, &c->iter)) return 1; break;
      case 'p': c->path = optarg; break;
      case 'y': c->noverify = true; break;
      case 'c': if (parse_unsigned(optarg, &c->batch)) return 1; break;
      case 't': c->burst = true; break;
      case 'm': c->use_bram = true; break;
      case 's': c->use_usm = true; break;
      case 'e': c->emulate = true; break;
      case 'h': usage(stdout); exit(0);
      default: return 1;
    }
  }
  if (optind != argc) return 1;
  if (!c->path) {
    fprintf(stderr, "Error parsing options: please input path to bitstream. Exiting! \n");
    exit(1);
  }
  if (c->dim < 1 || c->dim > 3 || c->iter < 1) return 1;
  return 0;
}

static void print_config(const config_t *c) {
  printf("\n------------------------------------------\n");
  printf("FFT CONFIGURATION: \n");
  printf("--------------------------------------------\n");
  printf("Type               : Complex to Complex\n");
  printf("Points             : %u%s \n", c->num, c->dim == 1 ? "" : c->dim == 2 ? "^2" : "^3");
  printf("Direction          : %s \n", c->inv ? "Backward" : "Forward");
  printf("Placement          : Out of Place\n");
  printf("Batch              : %u \n", c->batch);
  printf("Iterations         : %u \n", c->iter);
  printf("Transpose3D        : %s \n", c->use_bram ? "BRAM" : "DDR");
  printf("Burst Interleaving : %s \n", c->burst ? "Yes" : "No");
  printf("Emulation          : %s \n", c->emulate ? "Yes (runs on the GPU)" : "No");
  printf("USM Feature        : %s \n", c->use_usm ? "Yes" : "No");
  printf("--------------------------------------------\n\n");
}

/* ---- FP64 host FFT (verification) ---- */
static unsigned bitrev(unsigned x, unsigned bits) {
  unsigned r = 0;
  for (unsigned i = 0; i < bits; i++) r |= ((x >> i) & 1u) << (bits - 1 - i);
  return r;
}

/* in-place radix-2 FFT of n points at stride s; sign -1 forward, +1 backward
 * (unnormalised), twiddles from sin/cos in double */
static void fft_line(double *re, double *im, unsigned n, size_t s, int sign) {
  unsigned bits = 0;
  while ((1u << bits) < n) bits++;
  for (unsigned i = 0; i < n; i++) {
    const unsigned j = bitrev(i, bits);
    if (j > i) {
      double t = re[i * s]; re[i * s] = re[j * s]; re[j * s] = t;
      t = im[i * s]; im[i * s] = im[j * s]; im[j * s] = t;
    }
  }
  const double pi = 3.14159265358979323846;
  for (unsigned len = 2; len <= n; len <<= 1) {
    const unsigned half = len / 2;
    for (unsigned k = 0; k < half; k++) {
      const double a = sign * 2.0 * pi * (double)k / (double)len;
      const double wr = cos(a), wi = sin(a);
      for (unsigned b = 0; b < n; b += len) {
        const size_t p = (size_t)(b + k) * s, q = (size_t)(b + k + half) * s;
        const double xr = re[q] * wr - im[q] * wi;
        const double xi = re[q] * wi + im[q] * wr;
        re[q] = re[p] - xr; im[q] = im[p] - xi;
        re[p] += xr; im[p] += xi;
      }
    }
  }
}

/* SNR in dB of `got` (bit-reversed per block for 1D) against the FP64 FFT */
static double verify_snr(const float2 *inp, const float2 *got, const config_t *c) {
  const unsigned n = c->num;
  size_t sz = 1;
  for (unsigned d = 0; d < c->dim; d++) sz *= n;
  const size_t total = sz * c->batch;
  double *re = malloc(total * sizeof(double)), *im = malloc(total * sizeof(double));
  if (!re || !im) {
    free(re);
    free(im);
    return -1.0;
  }
  for (size_t i = 0; i < total; i++) {
    re[i] = inp[i].x;
    im[i] = inp[i].y;
  }
  const int sign = c->inv ? 1 : -1;
  for (unsigned b = 0; b < c->batch; b++) {
    double *r = re + b * sz, *m = im + b * sz;
    /* x (stride 1), then y (stride n), then z (stride n^2) */
    size_t stride = 1;
    for (unsigned d = 0; d < c->dim; d++) {
      const size_t block = stride * n;
      for (size_t o = 0; o < sz; o += block)
        for (size_t i = 0; i < stride; i++) fft_line(r + o + i, m + o + i, n, stride, sign);
      stride = block;
    }
  }
  unsigned bits = 0;
  while ((1u << bits) < n) bits++;
  double mag = 0.0, noise = 0.0;
  for (size_t i = 0; i < total; i++) {
    size_t j = i;
    if (c->dim == 1) j = (i / n) * n + bitrev((unsigned)(i % n), bits);
    const double dr = re[i] - got[j].x, di = im[i] - got[j].y;
    mag += re[i] * re[i] + im[i] * im[i];
    noise += dr * dr + di * di;
  }
  free(re);
  free(im);
  if (noise == 0.0) return INFINITY;
  return 10.0 * log10(mag / noise);
}

static fpga_t run(const config_t *c, const float2 *inp, float2 *out) {
  const unsigned n = c->num, inv = c->inv, burst = c->burst;
  fpga_t t = {0.0, 0.0, 0.0, 0.0, 0.0, false};
  switch (c->dim) {
    case 1:
      t = c->use_usm ? fftfpgaf_c2c_1d_svm(n, inp, out, inv, c->batch)
                     : fftfpgaf_c2c_1d(n, inp, out, inv, c->batch);
      break;
    case 2:
      if (c->use_bram && c->use_usm)
        t = fftfpgaf_c2c_2d_bram_svm(n, inp, out, inv, c->batch);
      else if (c->use_bram)
        t = fftfpgaf_c2c_2d_bram(n, inp, out, inv, burst, c->batch);
      else
        t = fftfpgaf_c2c_2d_ddr(n, inp, out, inv);
      break;
    case 3:
      if (c->use_bram)
        t = fftfpgaf_c2c_3d_bram(n, inp, out, inv, burst);
      else if (!c->use_usm && c->batch > 1)
        t = fftfpgaf_c2c_3d_ddr_batch(n, inp, out, inv, burst, c->batch);
      else if (c->use_usm)
        t = c->batch > 1 ? fftfpgaf_c2c_3d_ddr_svm_batch(n, inp, out, inv, c->batch)
                         : fftfpgaf_c2c_3d_ddr_svm(n, inp, out, inv, burst);
      else
        t = fftfpgaf_c2c_3d_ddr(n, inp, out, inv);
      break;
  }
  return t;
}

static void perf_measures(const config_t *c, const fpga_t *rt) {
  double ex = 0, rd = 0, wr = 0;
  for (unsigned i = 0; i < c->iter; i++) {
    ex += rt[i].exec_t;
    rd += rt[i].pcie_read_t;
    wr += rt[i].pcie_write_t;
  }
  ex /= c->iter;
  rd /= c->iter;
  wr /= c->iter;
  double vex = 0, vrd = 0, vwr = 0;
  for (unsigned i = 0; i < c->iter; i++) {
    vex += pow(rt[i].exec_t - ex, 2);
    vrd += pow(rt[i].pcie_read_t - rd, 2);
    vwr += pow(rt[i].pcie_write_t - wr, 2);
  }
  const double pts = c->batch * pow((double)c->num, (double)c->dim);
  const double gbs = pts * 8.0 / (ex * 1e-3) / 1e9;
  const double gflops =
      c->batch * c->dim * 5.0 * pow((double)c->num, (double)c->dim) * log2((double)c->num) /
      (ex * 1e-3) / 1e9;
  printf("\n\n------------------------------------------\n");
  printf("Measurements \n");
  printf("--------------------------------------------\n");
  printf("%s", c->iter > 1 ? "Average Measurements of iterations\n" : "");
  printf("PCIe Write          = %.4lfms\n", wr);
  printf("Kernel Execution    = %.4lfms\n", ex);
  printf("Kernel Exec/Batch   = %.4lfms\n", ex / c->batch);
  printf("PCIe Read           = %.4lfms\n", rd);
  printf("Total               = %.4lfms\n", ex + wr + rd);
  printf("Throughput          = %.4lfGFLOPS/s | %.4lf GB/s\n", gflops, gbs);
  if (c->iter > 1) {
    printf("\nDeviation of runtimes among iterations\n");
    printf("PCIe Write          = %.4lfms\n", sqrt(vwr / c->iter));
    printf("Kernel Execution    = %.4lfms\n", sqrt(vex / c->iter));
    printf("PCIe Read           = %.4lfms\n", sqrt(vrd / c->iter));
  }
}

int main(int argc, char **argv) {
  config_t c;
  if (parse_args(argc, argv, &c)) {
    usage(stderr);
    return 1;
  }
  print_config(&c);
  if (fpga_initialize("NVIDIA CUDA", c.path, c.use_usm) != 0) {
    fprintf(stderr, "FPGA initialization error\n");
    return EXIT_FAILURE;
  }
  size_t sz = c.batch;
  for (unsigned d = 0; d < c.dim; d++) sz *= c.num;
  float2 *inp = fftfpgaf_complex_malloc(sz * sizeof(float2));
  float2 *out = fftfpgaf_complex_malloc(sz * sizeof(float2));
  fpga_t *rt = calloc(c.iter, sizeof(fpga_t));
  if (!inp || !out || !rt) {
    fprintf(stderr, "host allocation of %zu points failed\n", sz);
    fpga_final();
    return EXIT_FAILURE;
  }
  for (size_t i = 0; i < sz; i++) {
    inp[i].x = (float)rand() / (float)RAND_MAX;
    inp[i].y = (float)rand() / (float)RAND_MAX;
  }
  int status = EXIT_SUCCESS;
  for (unsigned i = 0; i < c.iter; i++) {
    printf("%u: Calculating FFT - \n", i);
    rt[i] = run(&c, inp, out);
    if (!rt[i].valid) {
      fprintf(stderr, "Iter %u: invalid configuration or device failure\n", i);
      status = EXIT_FAILURE;
      break;
    }
    if (!c.noverify) {
      const double db = verify_snr(inp, out, &c);
      if (!(db > 120.0)) {
        printf("\tSignal to noise ratio on output sample: %f --> %s\n\n", db, "FAILED");
        fprintf(stderr, "Iter %u: result incorrect in comparison to the FP64 host FFT\n", i);
        status = EXIT_FAILURE;
        break;
      }
    }
  }
  fpga_final();
  if (status == EXIT_SUCCESS) perf_measures(&c, rt);
  free(inp);
  free(out);
  free(rt);
  return status;
}
