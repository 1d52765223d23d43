// ltimes_sym.h -- host logic of the mixed LTimes' octant-pair form (ltimes_stream.cu):
// the shapes the TMA-fed LTimes takes and the octant-pair table of an L matrix.  Plain
// C++, so the host tests compile it on their own.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <vector>

namespace kgb {

// the TMA-fed LTimes: directions in whole 32-direction chunks (at most 1024), 13 to 32 moments
inline bool ltimesStreamShape(int D, int M) { return D % 32 == 0 && D <= 1024 && M >= 13 && M <= 32; }

// Kernel::LTimes sums L(m, d) psi(d) over all directions (Kernel/LTimes.cpp:54-65).  Kripke's
// quadrature sets hold the octants one after another, the x sign running fastest, and a real
// spherical harmonic is even or odd under x -> -x: with 16 directions per octant the two
// octants of a 32-direction chunk are mirror images (in another order), and the partner's L
// column is the direction's times a sign that depends on the moment only (sets with 4
// directions per octant pair the chunk's halves across z instead; any such pairing serves).
// Found here from L alone (|L| equal to 1e-12 of the column's largest, one sign per moment
// over every chunk).  The table: per chunk the partner column (16..31) of each of its first
// 16 directions, then the moment of each of 32 slots (0-15: the moments of sign +1, 16-31:
// those of sign -1, ascending; -1 empty).
inline bool ltimesSymTable(const double *L, int D, int M, std::vector<int> &table) {
  table.clear();
  if (!ltimesStreamShape(D, M)) return false;
  const int nk = D / 32;
  std::vector<int> sign(M, 0), part((size_t)nk * 16, -1);
  for (int c = 0; c < nk; ++c) {
    bool used[16] = {};
    for (int b = 0; b < 16; ++b) {
      const double *la = L + (size_t)(32 * c + b) * M;
      double top = 0.0;
      for (int m = 0; m < M; ++m) top = std::max(top, std::fabs(la[m]));
      const double tol = 1e-12 * top;
      for (int b2 = 0; b2 < 16 && part[(size_t)c * 16 + b] < 0; ++b2) {
        if (used[b2]) continue;
        const double *lb = L + (size_t)(32 * c + 16 + b2) * M;
        bool ok = true;
        std::vector<int> sg(sign);
        for (int m = 0; m < M && ok; ++m) {
          if (std::fabs(std::fabs(lb[m]) - std::fabs(la[m])) > tol) ok = false;
          else if (std::fabs(la[m]) > tol) {
            const int t = (la[m] < 0) == (lb[m] < 0) ? 1 : -1;
            if (sg[m] == 0) sg[m] = t;
            else if (sg[m] != t) ok = false;
          }
        }
        if (!ok) continue;
        used[b2] = true;
        part[(size_t)c * 16 + b] = 16 + b2;
        sign = sg;
      }
      if (part[(size_t)c * 16 + b] < 0) return false;
    }
  }
  std::vector<int> even, odd;
  for (int m = 0; m < M; ++m) (sign[m] < 0 ? odd : even).push_back(m);
  if (even.size() > 16 || odd.size() > 16) return false;
  table = part;
  for (int k = 0; k < 32; ++k) {
    const std::vector<int> &v = k < 16 ? even : odd;
    const size_t i = (size_t)(k & 15);
    table.push_back(i < v.size() ? v[i] : -1);
  }
  return true;
}

}  // namespace kgb
