// fft_mix_4s.cu - the generic mixed-radix kernel's four-step forms
// (kernels/fft_mix_impl.cuh): the column pass with the W_N^(j1 k2) epilogue
// and the row pass with the transposed store, for factors that no two-stage
// instantiation covers.  A translation unit of its own so that it compiles
// beside the others.
#include "fft_mix_impl.cuh"

namespace fftgb {

void mix_fill_epi(MixEpiTable &t) {
  t[0][0][0] = k_mix<false, true, MIX_SMALL, 0, 1>;
  t[0][1][0] = k_mix<true, true, MIX_SMALL, 0, 1>;
  t[0][0][1] = k_mix<false, true, MIX_THREADS, 0, 1>;
  t[0][1][1] = k_mix<true, true, MIX_THREADS, 0, 1>;
  t[1][0][0] = k_mix<false, false, MIX_SMALL, 0, 2>;
  t[1][1][0] = k_mix<true, false, MIX_SMALL, 0, 2>;
  t[1][0][1] = k_mix<false, false, MIX_THREADS, 0, 2>;
  t[1][1][1] = k_mix<true, false, MIX_THREADS, 0, 2>;
}

}  // namespace fftgb
