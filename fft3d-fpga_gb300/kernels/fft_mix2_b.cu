// fft_mix2_b.cu - a third of the two-stage instantiations of the mixed-radix
// axis kernel (k_mix2, kernels/fft_mix_impl.cuh), complex, real-data
// and four-step forms; the thirds compile in parallel.
#include "fft_mix_impl.cuh"

namespace fftgb {

void mix2_fill_b(MixPairTable &t) {
  FFTGB_MIX2_PAIRS_B(FFTGB_MIX2_FILL)
}

void mix2_fill_real_b(MixPairRealTable &t) {
  FFTGB_MIX2_PAIRS_B(FFTGB_MIX2_FILL_REAL)
}

void mix2_fill_epi_b(MixPairEpiTable &t) {
  FFTGB_MIX2_PAIRS_B(FFTGB_MIX2_FILL_EPI)
}

}  // namespace fftgb
