"""The tensor-core combine's integer rounding (kripke_gb300/csrc/exact_round.h).

roundScaledOdd(h, l, scale) must equal, bit for bit, the two-double sum
h*2^(scale+32) + l*2^scale, both terms exact doubles, added once in IEEE
round-to-nearest-even.  The kernels pass |h| < 2^38 and |l| < 2^48; the test
covers |h| < 2^38 and |l| < 2^53 (where l is still an exact double).  The
header compiles for the host too; this test builds a small driver with g++
and checks random and constructed cases: ties and near-ties at every rounding
position, values on both sides of 2^63 (where the exact 64-bit path hands
over to the round-to-odd path), sign changes, and significand overflow on
rounding up.
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

static long long n = 0;

static int check(int64_t h, int64_t l, int e0) {
  const double hs = std::ldexp((double)h, e0 + 32), ls = std::ldexp((double)l, e0);
  if ((h != 0 && std::fabs(hs) < 2.2250738585072014e-308) || (l != 0 && std::fabs(ls) < 2.2250738585072014e-308))
    return 0;  // a term is not a normal number: outside the compared domain
  const double want = hs + ls;
  if (want != 0.0 && std::fabs(want) < 2.2250738585072014e-308) return 0;
  if (std::fabs(want) > 8.98846567431158e307) return 0;  // at the top binade the kernel takes its slow path
  bool ok = true;
  const double got = kgb::roundScaledOdd(h, l, e0, ok);
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
  const int64_t hlim = ((int64_t)1 << 38) - 1, llim = ((int64_t)1 << 53) - 1;
  std::uniform_int_distribution<int64_t> hd(-hlim, hlim), ld(-llim, llim);
  std::uniform_int_distribution<int> ex(-900, 900), hsh(0, 38), lsh(0, 53);
  int bad = 0;
  for (int i = 0; i < 3000000 && bad < 10; ++i) {
    // magnitudes spread over every bit length
    bad += check(hd(rng) >> hsh(rng), ld(rng) >> lsh(rng), ex(rng));
  }
  for (int i = 0; i < 300000 && bad < 10; ++i) {
    int64_t h = hd(rng) >> hsh(rng);
    if (h == 0) h = 1;
    // ties and near-ties: l at half an ulp of the h*2^32 part
    const int64_t ah = h < 0 ? -h : h;
    const int sh = 63 - __builtin_clzll((unsigned long long)ah) + 32 - 52;
    if (sh >= 1 && sh < 53) {
      const int64_t half = (int64_t)1 << (sh - 1);
      for (int d = -1; d <= 1; ++d) {
        bad += check(h, half + d, ex(rng));
        bad += check(h, -half + d, ex(rng));
        bad += check(h, 3 * half + d, ex(rng));
      }
    }
    // values near +-2^63, where the two paths meet
    for (int64_t hb : {((int64_t)1 << 31) - 1, ((int64_t)1 << 31), -((int64_t)1 << 31), -((int64_t)1 << 31) + 1,
                       -((int64_t)1 << 31) - 1})
      for (int64_t d : {(int64_t)0, (int64_t)-1, (int64_t)1, (int64_t)255, (int64_t)-256, (int64_t)128,
                        ((int64_t)1 << 32) - 1, -((int64_t)1 << 32), (int64_t)(ld(rng) >> 13)})
        bad += check(hb, d, ex(rng));
  }
  const int64_t hs_[] = {0, 1, -1, hlim, -hlim, (int64_t)1 << 31, -((int64_t)1 << 31), (int64_t)1 << 23};
  const int64_t ls_[] = {0, 1, -1, llim, -llim, 255, 256, -256, ((int64_t)1 << 32) - 1, -((int64_t)1 << 32)};
  for (int64_t h : hs_)
    for (int64_t l : ls_)
      for (int e0 : {-1000, -100, 0, 63, 500, 900}) bad += check(h, l, e0);
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
