// tc_selftest.cu - checks the tcgen05 operand layout, descriptors and TMEM
// read-back on the running GPU: one warpgroup computes D = A * B^T for a
// 128 x 32 A and a 32 x 32 B with half-precision inputs and FP32
// accumulators, which the host compares with an FP64 product.
#include <stdio.h>

#include <vector>

#include "fftfpga_ext.h"
#include "tc_core.cuh"

namespace fftgb {

__global__ void __launch_bounds__(128)
    k_tc_selftest(const float *A, const float *B, float *D, int bf16,
                  int *status) {
  __shared__ __align__(1024) uint8_t sa[128 * 32 * 2];
  __shared__ __align__(1024) uint8_t sb[32 * 32 * 2];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
#pragma unroll 4
  for (int k = 0; k < 32; k++) {
    const float a = A[tid * 32 + k];
    if (bf16)
      *(__nv_bfloat16 *)(sa + tc::core_off(tid, k, 32)) = __float2bfloat16_rn(a);
    else
      *(__half *)(sa + tc::core_off(tid, k, 32)) = __float2half_rn(a);
    if (tid < 32) {
      const float b = B[tid * 32 + k];
      if (bf16)
        *(__nv_bfloat16 *)(sb + tc::core_off(tid, k, 32)) = __float2bfloat16_rn(b);
      else
        *(__half *)(sb + tc::core_off(tid, k, 32)) = __float2half_rn(b);
    }
  }
  if (tid == 0) tc::mbar_init(&mbar, 1);
  if (warp == 0) {
    tc::tmem_alloc(&tslot, 32);
    tc::tmem_relinquish();
  }
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = tslot;
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_f16(bf16, 128, 32);
    for (int ks = 0; ks < 2; ks++) {
      const uint64_t ad = tc::smem_desc(tc::smem_u32(sa) + ks * 256, 128, 512);
      const uint64_t bd = tc::smem_desc(tc::smem_u32(sb) + ks * 256, 128, 512);
      tc::mma_f16(taddr, ad, bd, idesc, ks > 0 ? 1u : 0u);
    }
    tc::mma_commit(&mbar);
  }
  if (!tc::mbar_wait_bounded(&mbar, 0, 1u << 22)) atomicExch(status, 1);
  tc::fence_after_sync();
  float r[32];
  tc::tmem_ld32(taddr + ((uint32_t)(32 * warp) << 16), r);
#pragma unroll
  for (int c = 0; c < 32; c++) D[tid * 32 + c] = r[c];
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, 32);
}

}  // namespace fftgb

// Returns FFTGB_OK and the largest relative error of the tensor-core
// product (over all 128 x 32 outputs, relative to the largest |D|), or a
// status code.
extern "C" int fftgb_tc_selftest(int bf16, float *max_rel_err) {
  using namespace fftgb;
  std::vector<float> A(128 * 32), B(32 * 32), D(128 * 32);
  unsigned s = 12345u;
  auto rnd = [&s]() {
    s = s * 1664525u + 1013904223u;
    return (float)((int)((s >> 16) % 257) - 128) / 64.0f;  // exact in f16/bf16
  };
  for (float &v : A) v = rnd();
  for (float &v : B) v = rnd();
  float *dA = nullptr, *dB = nullptr, *dD = nullptr;
  int *dS = nullptr;
  int rc = FFTGB_OK;
  if (cudaMalloc(&dA, A.size() * 4) != cudaSuccess ||
      cudaMalloc(&dB, B.size() * 4) != cudaSuccess ||
      cudaMalloc(&dD, D.size() * 4) != cudaSuccess ||
      cudaMalloc(&dS, sizeof(int)) != cudaSuccess) {
    rc = FFTGB_ENOMEM;
  }
  if (!rc) {
    cudaMemcpy(dA, A.data(), A.size() * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(dB, B.data(), B.size() * 4, cudaMemcpyHostToDevice);
    cudaMemset(dD, 0, D.size() * 4);
    cudaMemset(dS, 0, sizeof(int));
    k_tc_selftest<<<1, 128>>>(dA, dB, dD, bf16, dS);
    if (cudaDeviceSynchronize() != cudaSuccess) rc = FFTGB_ECUDA;
  }
  int status = 0;
  if (!rc) {
    cudaMemcpy(D.data(), dD, D.size() * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(&status, dS, sizeof(int), cudaMemcpyDeviceToHost);
    if (status) rc = FFTGB_ETIMEOUT;
  }
  if (!rc) {
    double maxd = 0.0, maxe = 0.0;
    for (int m = 0; m < 128; m++)
      for (int n = 0; n < 32; n++) {
        double ref = 0.0;
        for (int k = 0; k < 32; k++) ref += (double)A[m * 32 + k] * B[n * 32 + k];
        maxd = fmax(maxd, fabs(ref));
        maxe = fmax(maxe, fabs(ref - D[m * 32 + n]));
      }
    if (max_rel_err) *max_rel_err = (float)(maxe / (maxd > 0 ? maxd : 1.0));
  }
  if (dA) cudaFree(dA);
  if (dB) cudaFree(dB);
  if (dD) cudaFree(dD);
  if (dS) cudaFree(dS);
  return rc;
}
