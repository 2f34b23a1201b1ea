// tables.h - host-side twiddle tables (evaluated in FP64, rounded once).
//
// Two layouts:
//  * w_table: W_n^(i*step) for i < count (natural order), used for the
//    four-step and y-split twiddles;
//  * stage_table: the per-stage blocks a Stockham plan of length L with E
//    points per thread reads (layout of Stock<L, E>::stage_off in
//    kernels/fft_core.cuh): for stages s >= 1, W_{NS*R}^(jr*k) at [k][jr].
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include <vector>

namespace fftgb {

inline float2 w_value(long long n, long long m) {
  m %= n;
  double s, c;
  sincos(-2.0 * M_PI * ((double)m / (double)n), &s, &c);
  float2 w;
  w.x = (float)c;
  w.y = (float)s;
  return w;
}

inline void w_table(std::vector<float2> &v, long long n, long long count,
                    long long step) {
  for (long long i = 0; i < count; i++) v.push_back(w_value(n, i * step));
}

// Stage geometry of Stock<L, E> computed at run time (same rules as the
// compile-time template).
struct StageGeo {
  int L, E, LOG, LOGE, NSTG;
  StageGeo(int l, int e) : L(l) {
    E = e < l ? e : l;
    LOG = 0;
    while ((1 << LOG) < L) LOG++;
    LOGE = 0;
    while ((1 << LOGE) < E) LOGE++;
    NSTG = LOGE ? (LOG + LOGE - 1) / LOGE : 1;
  }
  int radix(int s) const {
    return (s < NSTG - 1) ? E : (1 << (LOG - LOGE * (NSTG - 1)));
  }
  int ns(int s) const { return 1 << (LOGE * s); }
};

inline size_t stage_table_entries(int L, int E) {
  StageGeo g(L, E);
  size_t n = 0;
  for (int s = 1; s < g.NSTG; s++) n += (size_t)g.radix(s) * g.ns(s);
  return n;
}

// Appends the stage table of Stock<L, E> to v.
inline void stage_table(std::vector<float2> &v, int L, int E) {
  StageGeo g(L, E);
  for (int s = 1; s < g.NSTG; s++) {
    const int R = g.radix(s), NS = g.ns(s);
    for (int k = 0; k < R; k++)
      for (int jr = 0; jr < NS; jr++)
        v.push_back(w_value(L, (long long)jr * k * (L / (NS * R))));
  }
}

}  // namespace fftgb
