"""The tensor-core combine's integer rounding (kripke_gb300/csrc/exact_round.h).

roundScaled32(h, l, scale) must equal, bit for bit, the two-double sum
h*2^(scale+32) + l*2^scale, both terms exact doubles, added once in IEEE
round-to-nearest-even (the kernels pass |h| < 2^41, |l| < 2^49; the test also
covers wider h, up to 2^52, where the significand lies in the high word alone).  The header compiles for the host too; this test builds
a small driver with g++ and checks random and constructed cases (ties, carries
across the 64-bit boundary, sign changes, mantissa overflow on rounding up).
"""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DRIVER = r"""
#include "exact_round.h"
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

template <int SHIFT>
static int check(int64_t h, int64_t l, int e0, long long &n) {
  const double hs = std::ldexp((double)h, e0 + SHIFT), ls = std::ldexp((double)l, e0);
  if ((h != 0 && std::fabs(hs) < 2.2250738585072014e-308) || (l != 0 && std::fabs(ls) < 2.2250738585072014e-308))
    return 0;  // a term is not a normal number: outside the compared domain
  const double want = hs + ls;
  if (want != 0.0 && std::fabs(want) < 2.2250738585072014e-308) return 0;
  bool ok = true;
  const double got = kgb::roundScaled32(h, l, e0, ok);
  ++n;
  uint64_t a, b;
  std::memcpy(&a, &got, 8);
  std::memcpy(&b, &want, 8);
  if (!ok || a != b) {
    std::printf("MISMATCH shift=%d h=%lld l=%lld e0=%d got=%.17g want=%.17g ok=%d\n", SHIFT, (long long)h,
                (long long)l, e0, got, want, (int)ok);
    return 1;
  }
  return 0;
}

template <int SHIFT>
static int run(int hbits, int lbits, long long &n) {
  std::mt19937_64 rng(20261204 + SHIFT);
  const int64_t hlim = ((int64_t)1 << hbits) - 1, llim = ((int64_t)1 << lbits) - 1;
  std::uniform_int_distribution<int64_t> hd(-hlim, hlim), ld(-llim, llim);
  std::uniform_int_distribution<int> ex(-900, 900), hsh(0, hbits), lsh(0, lbits);
  int bad = 0;
  for (int i = 0; i < 2000000 && bad < 10; ++i) {
    // magnitudes spread over every bit length
    const int64_t h = hd(rng) >> hsh(rng), l = ld(rng) >> lsh(rng);
    bad += check<SHIFT>(h, l, ex(rng), n);
  }
  for (int i = 0; i < 200000 && bad < 10; ++i) {
    // ties and near-ties: l at exactly half an ulp of the h*2^SHIFT part
    int64_t h = hd(rng) >> hsh(rng);
    if (h == 0) h = 1;
    const int p = 63 - __builtin_clzll((unsigned long long)(h < 0 ? -h : h)) + SHIFT;
    const int sh = p - 52;
    if (sh >= 1 && sh < lbits) {
      const int64_t half = (int64_t)1 << (sh - 1);
      for (int d = -1; d <= 1; ++d) {
        bad += check<SHIFT>(h, half + d, ex(rng), n);
        bad += check<SHIFT>(h, -half + d, ex(rng), n);
        bad += check<SHIFT>(h, 3 * half + d, ex(rng), n);
      }
    }
  }
  const int64_t hs_[] = {0, 1, -1, hlim, -hlim, (int64_t)1 << (hbits - 1), -((int64_t)1 << (hbits - 1))};
  const int64_t ls_[] = {0, 1, -1, llim, -llim, (int64_t)1 << SHIFT, -((int64_t)1 << SHIFT), ((int64_t)1 << SHIFT) - 1};
  for (int64_t h : hs_)
    for (int64_t l : ls_)
      for (int e0 : {-1000, -100, 0, 63, 500, 900}) bad += check<SHIFT>(h, l, e0, n);
  return bad;
}

int main() {
  long long n = 0;
  int bad = run<32>(41, 49, n) + run<32>(52, 49, n) + run<32>(20, 49, n);
  std::printf("checked %lld mismatches %d\n", n, bad);
  return bad != 0;
}
"""


def test_round_scaled_matches_two_double_sum(tmp_path):
    src = tmp_path / "drv.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "drv"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "kripke_gb300", "csrc"),
                    str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], stdout=subprocess.PIPE, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:]
    assert "mismatches 0" in r.stdout
