// fft3d_fused_cfg.cuh - tile geometry of the two-pass 3D kernels
// (fft3d_fused.cu; the TMA-fed forms in fft3d_fused_tma.cu size their own).
#pragma once

#include "fft_core.cuh"

namespace fftgb {

// E: points per thread (16; 8 halves every thread's serial chain for the
// latency-bound small grids)
template <int NX, int NJ, int E_ = 16>
struct XyCfg {
  static constexpr int E = E_;
  using CX = Stock<NX, E>;
  using CJ = Stock<NJ, E>;
  static constexpr int THREADS = NJ * NX / E;
  static constexpr int SMEM = NJ * NX * (int)sizeof(float2);
  static_assert(NX >= E && NJ >= 2 && NX * NJ >= E * 32, "tile too small");
  static_assert(THREADS <= 1024, "tile too large");
};

template <int NZ, int R, int X, int E_ = 16>
struct RzCfg {
  static constexpr int E = E_;
  using CZ = Stock<NZ, E>;
  static constexpr int THREADS = X * R * NZ / E;
  // A half-warp covers X columns of 16/X residue blocks; offsetting block
  // k2 by k2*X elements puts those blocks in disjoint shared-memory banks.
  static constexpr int KS = NZ * X + (X < 16 ? X : 0);  // block stride
  static constexpr int SMEM = R * KS * (int)sizeof(float2);
  static_assert(THREADS <= 1024, "tile too large");
  static_assert(E % R == 0, "R must divide 16");
};

}  // namespace fftgb
