// fft_mix2_a.cu - a third of the two-stage instantiations of the mixed-radix
// axis kernel (k_mix2, kernels/fft_mix_impl.cuh), complex, real-data
// and four-step forms; the thirds compile in parallel.
#include "fft_mix_impl.cuh"

namespace fftgb {

void mix2_fill_a(MixPairTable &t) {
  FFTGB_MIX2_PAIRS_A(FFTGB_MIX2_FILL)
}

void mix2_fill_real_a(MixPairRealTable &t) {
  FFTGB_MIX2_PAIRS_A(FFTGB_MIX2_FILL_REAL)
}

void mix2_fill_epi_a(MixPairEpiTable &t) {
  FFTGB_MIX2_PAIRS_A(FFTGB_MIX2_FILL_EPI)
}

}  // namespace fftgb
