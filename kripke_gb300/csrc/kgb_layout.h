// kgb_layout.h -- host-side index conventions shared by the C ABI and the
// problem generator: the six nestings and the single-rank partition spaces.
//
// Nesting rule (src/Kripke/VarTypes.h:67-101, Core/VarLayout.h:118-170): a
// field chunk's index types are ordered by their position in the nesting's
// order list (ties keep argument order); the first has the longest stride.
// Subdomains (Core/PartitionSpace.cpp:82-92,246-273): row-major over
// (P, Q, Rx, Ry, Rz); a field over a space has one chunk per subdomain of that
// space, in space-index order (Core/DomainVar.cpp:15-39).
#pragma once

#include <stdint.h>

#include <utility>

namespace kgb {

enum Idx { I_LONG, I_DIM, I_MAT, I_DIR, I_LEG, I_MOM, I_GGRP, I_GRP, I_ZONE, I_ZK, I_ZJ, I_ZI, I_MIX };

inline const Idx *nestOrder(int layout) {
  static const Idx kNest[6][13] = {
      {I_LONG, I_DIM, I_MAT, I_DIR, I_LEG, I_MOM, I_GGRP, I_GRP, I_ZONE, I_ZK, I_ZJ, I_ZI, I_MIX},  // DGZ
      {I_LONG, I_DIM, I_MAT, I_DIR, I_LEG, I_MOM, I_ZONE, I_ZK, I_ZJ, I_ZI, I_GGRP, I_GRP, I_MIX},  // DZG
      {I_LONG, I_DIM, I_MAT, I_GGRP, I_GRP, I_DIR, I_LEG, I_MOM, I_ZONE, I_ZK, I_ZJ, I_ZI, I_MIX},  // GDZ
      {I_LONG, I_DIM, I_MAT, I_GGRP, I_GRP, I_ZONE, I_ZK, I_ZJ, I_ZI, I_MIX, I_DIR, I_LEG, I_MOM},  // GZD
      {I_LONG, I_DIM, I_MAT, I_ZONE, I_ZK, I_ZJ, I_ZI, I_MIX, I_DIR, I_LEG, I_MOM, I_GGRP, I_GRP},  // ZDG
      {I_LONG, I_DIM, I_MAT, I_ZONE, I_ZK, I_ZJ, I_ZI, I_MIX, I_GGRP, I_GRP, I_DIR, I_LEG, I_MOM},  // ZGD
  };
  return kNest[layout];
}

inline void nestStrides(int layout, int n, const Idx *types, const int64_t *dims, int64_t *strides) {
  const Idx *order = nestOrder(layout);
  int pos[4], ord[4];
  for (int i = 0; i < n; ++i) {
    pos[i] = 0;
    for (int k = 0; k < 13; ++k)
      if (order[k] == types[i]) pos[i] = k;
    ord[i] = i;
  }
  for (int i = 1; i < n; ++i)  // insertion sort: equal keys keep argument order
    for (int k = i; k > 0 && pos[ord[k]] < pos[ord[k - 1]]; --k) std::swap(ord[k], ord[k - 1]);
  int64_t s = 1;
  for (int k = n - 1; k >= 0; --k) {
    strides[ord[k]] = s;
    s *= dims[ord[k]];
  }
}

enum Space { S_P, S_Q, S_RX, S_RY, S_RZ, S_R, S_PR, S_PQR, S_NULL };

struct Decomp {
  int SP = 1, SQ = 1, Sx = 1, Sy = 1, Sz = 1;
  int num() const { return SP * SQ * Sx * Sy * Sz; }
  void coord(int s, int c[5]) const {
    c[4] = s % Sz; s /= Sz;
    c[3] = s % Sy; s /= Sy;
    c[2] = s % Sx; s /= Sx;
    c[1] = s % SQ;
    c[0] = s / SQ;
  }
  int sdomOf(const int c[5]) const { return (((c[0] * SQ + c[1]) * Sx + c[2]) * Sy + c[3]) * Sz + c[4]; }
  int chunks(Space s) const {
    switch (s) {
      case S_P: return SP; case S_Q: return SQ; case S_RX: return Sx; case S_RY: return Sy; case S_RZ: return Sz;
      case S_R: return Sx * Sy * Sz; case S_PR: return SP * Sx * Sy * Sz; case S_PQR: return num();
      default: return 1;
    }
  }
  // coordinates (p, q, x, y, z) of a space chunk; projected-out coordinates are 0
  void chunkCoord(Space s, int ch, int c[5]) const {
    for (int k = 0; k < 5; ++k) c[k] = 0;
    switch (s) {
      case S_P: c[0] = ch; break;
      case S_Q: c[1] = ch; break;
      case S_RX: c[2] = ch; break;
      case S_RY: c[3] = ch; break;
      case S_RZ: c[4] = ch; break;
      case S_R: c[4] = ch % Sz; ch /= Sz; c[3] = ch % Sy; c[2] = ch / Sy; break;
      case S_PR: c[4] = ch % Sz; ch /= Sz; c[3] = ch % Sy; ch /= Sy; c[2] = ch % Sx; c[0] = ch / Sx; break;
      case S_PQR: coord(ch, c); break;
      default: break;
    }
  }
  int rIndex(const int c[5]) const { return (c[2] * Sy + c[3]) * Sz + c[4]; }
};

}  // namespace kgb
