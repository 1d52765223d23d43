"""Host logic of the mixed LTimes' octant-pair form (kripke_gb300/csrc/ltimes_sym.h).

ltimesSymTable finds, from L alone, the partner of each of a 32-direction chunk's first 16
directions among the other 16 (|L| equal column for column, one sign per moment over all
chunks) and the moment slots of the kernel's lane groups.  On the oracle's L and L+ tables
(the generator restated from Kripke's Generate/Quadrature.cpp): the sets with 16 directions per
octant (8x16) and with 4 (4x8) have the structure, 8x12, 8x24 and 16x16 do not; where it is
found, sum_b L(m,b) (psi(b) + s_m psi(b')) over the table equals L psi to FP64 rounding.  The
driver is compiled with g++ from the header the library uses.
"""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DRIVER = r"""
#include "ltimes_sym.h"
#include <cstdio>
#include <cstdlib>
int main(int argc, char **argv) {
  const int D = std::atoi(argv[2]), M = std::atoi(argv[3]);
  std::vector<double> L((size_t)D * M);
  FILE *f = std::fopen(argv[1], "rb");
  if (!f || std::fread(L.data(), sizeof(double), L.size(), f) != L.size()) return 2;
  std::fclose(f);
  std::vector<int> t;
  const bool ok = kgb::ltimesSymTable(L.data(), D, M, t);
  std::printf("%d\n", ok ? 1 : 0);
  for (int v : t) std::printf("%d ", v);
  std::printf("\n");
  return 0;
}
"""


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    d = tmp_path_factory.mktemp("symtab")
    src = d / "drv.cpp"
    src.write_text(DRIVER)
    exe = d / "drv"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "kripke_gb300", "csrc"), str(src), "-o",
                    str(exe)], check=True)
    return d, exe


def table_of(driver, L, D, M):
    d, exe = driver
    path = d / "L.bin"
    np.ascontiguousarray(L, dtype=np.float64).tofile(path)
    out = subprocess.run([str(exe), str(path), str(D), str(M)], stdout=subprocess.PIPE, text=True,
                         check=True).stdout.split("\n")
    return out[0].strip() == "1", [int(x) for x in out[1].split()]


@pytest.mark.parametrize("quad,legendre,found", [((8, 16), 4, True), ((8, 16), 3, True), ((4, 8), 4, True),
                                                 ((8, 12), 4, False), ((8, 24), 4, False), ((16, 16), 4, False),
                                                 ((8, 16), 2, False)])
def test_octant_pair_table(oracle, driver, quad, legendre, found):
    p = oracle.Problem(zones=(3, 3, 3), groups=1, quad=quad, legendre=legendre, gset=1, dset=8)
    D, M = quad[0] * quad[1], (legendre + 1) ** 2
    rng = np.random.default_rng(7)
    for name in ("ell", "ell_plus"):
        L = p.get(name).reshape(D, M)  # [direction][moment]
        ok, t = table_of(driver, L, D, M)
        assert ok == found, name
        if not ok:
            assert t == []
            continue
        nk = D // 32
        part = np.array(t[:nk * 16]).reshape(nk, 16)
        slot = np.array(t[nk * 16:])
        assert len(slot) == 32 and sorted(x for x in slot if x >= 0) == list(range(M))
        for c in range(nk):
            assert sorted(part[c]) == list(range(16, 32))
        psi = rng.uniform(-1.0, 2.0, (4, D))
        want = psi @ L
        got = np.zeros_like(want)
        for c in range(nk):
            for b in range(16):
                d, dp = 32 * c + b, 32 * c + part[c, b]
                for s, m in enumerate(slot):
                    if m >= 0:
                        got[:, m] += L[d, m] * (psi[:, d] + (1.0 if s < 16 else -1.0) * psi[:, dp])
        assert np.max(np.abs(got - want)) <= 1e-13 * np.max(np.abs(want)), name


def test_octant_pair_table_rejects_broken_symmetry(oracle, driver):
    p = oracle.Problem(zones=(3, 3, 3), groups=1, quad=(8, 16), legendre=4, gset=1, dset=8)
    L = p.get("ell").reshape(128, 25).copy()
    assert table_of(driver, L, 128, 25)[0]
    L[37, 5] *= 1.0 + 1e-9  # one entry off its mirror's magnitude
    assert not table_of(driver, L, 128, 25)[0]
    L = p.get("ell").reshape(128, 25).copy()
    L[16:32, 3] = np.abs(L[16:32, 3])  # moment 3 loses its sign pattern in the first chunk only
    L[:16, 3] = np.abs(L[:16, 3])
    ok, _ = table_of(driver, L, 128, 25)
    assert not ok
