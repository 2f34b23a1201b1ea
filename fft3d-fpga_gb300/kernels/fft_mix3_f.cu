// fft_mix3_f.cu - a sixth of the three-stage instantiations of the
// mixed-radix axis kernel (k_mix3, kernels/fft_mix_impl.cuh), complex,
// real-data and four-step forms; the sixths compile in parallel.
#include "fft_mix_impl.cuh"

namespace fftgb {

void mix3_fill_f(MixTripleTable &t) {
  FFTGB_MIX3_TRIPLES_F(FFTGB_MIX3_FILL)
}

void mix3_fill_real_f(MixTripleRealTable &t) {
  FFTGB_MIX3_TRIPLES_F(FFTGB_MIX3_FILL_REAL)
}

void mix3_fill_epi_f(MixTripleEpiTable &t) {
  FFTGB_MIX3_TRIPLES_F(FFTGB_MIX3_FILL_EPI)
}

}  // namespace fftgb
