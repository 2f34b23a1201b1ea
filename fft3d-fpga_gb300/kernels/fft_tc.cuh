// fft_tc.cuh - tensor-core split-precision axis passes (fft_tc.cu).
#pragma once

#include <cuda_runtime.h>

#include "fft_pass.cuh"

namespace fftgb {

cudaError_t tc_kernels_init();
// a tensor-core kernel exists for length 2^log_l (256 and 512)
bool tc_available(int log_l);
// mode 1: split FP16 (3 products), mode 2: split BF16 (6 products)
cudaError_t launch_rows_tc(int log_l, int mode, const RowsArgs &a, cudaStream_t s);
cudaError_t launch_cols_tc(int log_l, int mode, const ColsArgs &a, cudaStream_t s);
// 1 if a tensor-core wait gave up since the last call (then cleared)
int tc_status_and_clear();
cudaError_t tc_expire_wait(unsigned polls);

}  // namespace fftgb
