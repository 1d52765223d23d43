"""The tensor-core combine's integer rounding (kripke_gb300/csrc/exact_round.h).

roundScaled(h, l, e0) must equal, bit for bit, the two-double sum it replaces:
h*2^(e0-35) + l*2^(e0-63), both terms exact doubles, added once in IEEE
round-to-nearest-even.  The header compiles for the host too; this test builds
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

static int check(int64_t h, int64_t l, int e0, long long &n) {
  const double hs = std::ldexp((double)h, e0 - 35), ls = std::ldexp((double)l, e0 - 63);
  if ((h != 0 && std::fabs(hs) < 2.2250738585072014e-308) || (l != 0 && std::fabs(ls) < 2.2250738585072014e-308))
    return 0;  // a term is not a normal number: outside the compared domain
  const double want = hs + ls;
  if (want != 0.0 && std::fabs(want) < 2.2250738585072014e-308) return 0;
  bool ok = true;
  const double got = kgb::roundScaled(h, l, e0, ok);
  ++n;
  uint64_t a, b;
  std::memcpy(&a, &got, 8);
  std::memcpy(&b, &want, 8);
  if (!ok || a != b) {
    std::printf("MISMATCH h=%lld l=%lld e0=%d got=%.17g want=%.17g ok=%d\n", (long long)h, (long long)l, e0, got,
                want, (int)ok);
    return 1;
  }
  return 0;
}

int main() {
  std::mt19937_64 rng(20261204);
  const int64_t lim = (1ll << 47) - 1;
  std::uniform_int_distribution<int64_t> full(-lim, lim);
  std::uniform_int_distribution<int> ex(-900, 900), bits(0, 47);
  long long n = 0;
  int bad = 0;
  for (int i = 0; i < 2000000 && bad < 10; ++i) {
    // magnitudes spread over every bit length
    int64_t h = full(rng) >> bits(rng), l = full(rng) >> bits(rng);
    bad += check(h, l, ex(rng), n);
  }
  for (int i = 0; i < 200000 && bad < 10; ++i) {
    // ties and near-ties: l's low bits at exactly half an ulp of the h*2^28 part
    int64_t h = full(rng) >> bits(rng);
    if (h == 0) h = 1;
    const int p = 63 - __builtin_clzll((unsigned long long)(h < 0 ? -h : h)) + 28;
    const int sh = p - 52;
    if (sh >= 1 && sh < 47) {
      int64_t half = (int64_t)1 << (sh - 1);
      for (int d = -1; d <= 1; ++d) {
        bad += check(h, half + d, ex(rng), n);
        bad += check(h, -half + d, ex(rng), n);
        bad += check(h, 3 * half + d, ex(rng), n);
      }
    }
  }
  const int64_t hs_[] = {0, 1, -1, lim, -lim, (int64_t)1 << 46, -((int64_t)1 << 46)};
  const int64_t ls_[] = {0, 1, -1, lim, -lim, (int64_t)1 << 28, -((int64_t)1 << 28), ((int64_t)1 << 28) - 1};
  for (int64_t h : hs_)
    for (int64_t l : ls_)
      for (int e0 : {-1000, -100, 0, 63, 500, 1000}) bad += check(h, l, e0, n);
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
