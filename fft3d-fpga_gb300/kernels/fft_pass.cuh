// fft_pass.cuh - argument blocks and launchers of the generic axis passes.
#pragma once

#include <cuda_runtime.h>

namespace fftgb {

// FFT of length L along the contiguous axis, `nrows` rows of L points.
struct RowsArgs {
  const float2 *in;
  float2 *out;
  long long nrows;
  const float2 *tw;  // W_L^m, m < L
  float scale;
  int swap_io;   // 1: inverse (real/imag swap on load and store)
  int in_mode;   // 0: natural, 1: load position bitrev(n) (adjoint of mode 1)
  int out_mode;  // 0: natural, 1: bit-reversed within the row,
                 // 2: as 1 and rows permuted by bitrev over rows_log bits,
                 // 3: natural within the row, rows of grids [b][z][y] moved
                 //    to the y-blocked layout [b][y/8][z][y%8] (blk_*)
                 // 4: transposed within transforms of 2^rows_log rows: row
                 //    (b, r) puts element k at (b*L + k)*2^rows_log + r (the
                 //    four-step's output order; see rows_transposed_supported)
  int rows_log;
  int blk_lny = 0;  // out_mode 3: log2 ny (ny >= 8) and log2 nz
  int blk_lnz = 0;
};

// FFT of length L along a strided axis: data [outer][L][inner], one FFT per
// (outer, inner) column, `ncols` = outer * inner.
struct ColsArgs {
  const float2 *in;
  float2 *out;
  long long ncols;
  long long inner;
  const float2 *tw;  // W_L^m, m < L
  // optional four-step twiddle on output k of column c = col % inner:
  // W_{inner*L}^{c*k} = tw4_lo[e & mask] * tw4_hi[e >> tw4_bits]
  const float2 *tw4_lo;
  const float2 *tw4_hi;
  int tw4_bits;
  float scale;
  int swap_io;
  int out_mode;  // 0: same layout (in place capable), 1: transposed, output
                 // (col, k) at col*L + k (out of place only)
  int tw_in = 0;  // 1: the twiddle multiplies input n of column c by
                  // W^((c >> tw_shift)*n) (tables tw4_*) before the transform,
                  // not the outputs: the four-step's W_{inner*L}^(c*n)
                  // (tw_shift 0) or a 2D plan's W_ny^(k1*r), k1 = c / nx
  int tw_shift = 0;
  // >= 0 (k_cols_tma only): the input is in the y-blocked layout
  // [b][L/8][nz][8][inner] of grids [b][nz][L][inner] (L = ny, inner = nx)
  // with nz = 2^blk_lnz, read by 5D tensor copies; the output is natural
  int blk_lnz = -1;
};

// Launch helpers; return cudaSuccess or the launch error.  `log_l` in 1..12.
// pdl: programmatic dependent launch after the previous kernel of stream s
cudaError_t launch_rows(int log_l, const RowsArgs &a, cudaStream_t s, bool pdl = false);
cudaError_t launch_cols(int log_l, const ColsArgs &a, cudaStream_t s, bool pdl = false);

// out[b*n + j] = in[b*n + bitrev(j)] for `count` blocks of n points.
cudaError_t launch_bitrev_gather(const float2 *in, float2 *out, long long n,
                                 int log_n, long long count, cudaStream_t s);

// One-time kernel attribute setup (dynamic shared memory limits).
cudaError_t pass_kernels_init();

// Sets the dynamic shared-memory limits of every pass kernel on the current
// device (no allocation); the *_on launchers need only this.
cudaError_t pass_kernels_set_attributes_current_device();
cudaError_t launch_rows_on(int log_l, const RowsArgs &a, cudaStream_t s);
cudaError_t launch_cols_on(int log_l, const ColsArgs &a, cudaStream_t s);

// persistent column pass fed by TMA tensor copies into two alternating
// buffers (fft_pass_tma.cu): L in {128, 256, 512}, out_mode 0, no four-step
// twiddle; cudaErrorNotSupported otherwise (or without a tensor-map
// encoder), cudaErrorMisalignedAddress for an input not 16-byte aligned
cudaError_t cols_tma_init();
bool cols_tma_supported(int log_l, long long ncols, long long inner);
cudaError_t launch_cols_tma(int log_l, const ColsArgs &a, cudaStream_t s, bool pdl = false);
// 1 if a TMA completion wait gave up since the last call (clears it), -1 on
// a CUDA error
int cols_tma_status_and_clear();
// sets the status word through the give-up path of a bounded wait (test hook)
cudaError_t cols_tma_expire_wait(unsigned polls);

// out_mode 4 exists for rows of length 2^log_l whose CTAs hold 8-32 rows
// (64 <= L <= 1024) and transforms of 2^rows_log rows, a multiple of that.
bool rows_transposed_supported(int log_l, int rows_log);

// Shared-memory bytes and threads per CTA, for reporting.
int rows_threads(int log_l);
int cols_threads(int log_l);

}  // namespace fftgb
