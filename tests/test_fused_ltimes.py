"""The LTimes epilogue fused into the mixed form's sweep (option fused_ltimes; sweep.cu, LTF).

Inside one solve, the sweep of every iteration but the last adds the next iteration's moments
phi = L psi (Kernel::LTimes, src/Kripke/Kernel/LTimes.cpp:54-65) slice by slice -- each block
sums its subdomain's directions per (zone, group, moment) and adds the sum with FP32
reductions -- and the next iteration runs no LTimes (the solver loop of
src/Kripke/SteadyStateSolver.cpp:53-99).  The order in which the subdomains' sums meet is not
fixed, so results are compared with tolerances: against the FP64 oracle as every mixed solve is
(phi 2-norm ratio 1e-6, largest entry 2e-6, particle counts 2e-6), and against the same solve
without the epilogue.  phi after the solve is L of the psi the last iteration started from, as
without the epilogue.
"""
import numpy as np
import pytest

from tests.test_gpu_parity import pair

pytestmark = pytest.mark.gpu

CASES = [
    dict(zones=(12, 10, 8), groups=32, quad=(4, 8), legendre=4),                      # 128 chains per subdomain
    dict(zones=(10, 8, 9), groups=16, quad=(8, 16), legendre=3, geometry=1, scatter=1),  # 256 chains
    dict(zones=(8, 9, 10), groups=64, quad=(4, 8), legendre=2, gset=2, zsets=(2, 1, 2)),  # group and zone sets
    dict(zones=(9, 8, 7), groups=8, quad=(8, 16), legendre=4, layout="GZD", dset=8),
]


@pytest.mark.parametrize("kw", CASES)
def test_fused_ltimes_solve(oracle, kgb, kw):
    p, ctx = pair(oracle, kgb, precision=kgb.MIXED, **kw)
    want_parts = p.solve(8)
    want = p.get("phi")
    ctx.set_option("fused_ltimes", 1)
    assert ctx.get_option("fused_ltimes_active") == 1
    parts = ctx.solve(8)
    fused_phi, fused_psi = ctx.download("phi"), ctx.download("psi")
    ctx.set_option("fused_ltimes", 0)
    plain = ctx.solve(8)
    plain_phi, plain_psi = ctx.download("phi"), ctx.download("psi")
    e = np.linalg.norm(fused_phi - want) / np.linalg.norm(want)
    m = np.max(np.abs(fused_phi - want)) / np.max(np.abs(want))
    print("fused LTimes: phi error vs FP64 (2-norm / max-abs) %.3e / %.3e" % (e, m))
    assert e <= 1e-6 and m <= 2e-6
    np.testing.assert_allclose(parts, want_parts, rtol=2e-6)
    np.testing.assert_allclose(parts, plain, rtol=2e-6)
    assert np.linalg.norm(fused_psi - plain_psi) <= 2e-6 * np.linalg.norm(plain_psi)
    assert np.linalg.norm(fused_phi - plain_phi) <= 2e-6 * np.linalg.norm(plain_phi)
    ctx.close()


def test_fused_ltimes_one_iteration_and_graph(kgb):
    """A one-iteration solve fuses nothing (its LTimes is the plain kernel's, bit for bit); a
    replayed solve graph gives the eager solve's results within rounding."""
    kw = dict(zones=(12, 10, 8), groups=32, quad=(4, 8), legendre=4)
    a, b = kgb.Context(0), kgb.Context(0)
    for c in (a, b):
        c.generate(precision=kgb.MIXED, **kw)
    a.set_option("fused_ltimes", 1)
    assert a.solve(1) == b.solve(1)
    np.testing.assert_array_equal(a.download("phi"), b.download("phi"))
    np.testing.assert_array_equal(a.download("psi"), b.download("psi"))
    a.set_option("graph", 0)
    eager = a.solve(6)
    a.set_option("graph", 1)
    replay = a.solve(6)
    assert a.get_option("graph_active") == 1
    np.testing.assert_allclose(replay, eager, rtol=2e-6)
    a.close(); b.close()


def test_fused_ltimes_inactive_where_it_does_not_apply(kgb):
    c = kgb.Context(0)
    c.generate(precision=kgb.FP64, zones=(6, 6, 6), groups=32, quad=(4, 8), legendre=2)
    c.set_option("fused_ltimes", 1)
    assert c.get_option("fused_ltimes_active") == 0  # FP64
    c.close()
    c = kgb.Context(0)
    c.generate(precision=kgb.MIXED, zones=(6, 6, 6), groups=12, quad=(4, 8), legendre=2)
    c.set_option("fused_ltimes", 1)
    assert c.get_option("fused_ltimes_active") == 0  # 48 chains per subdomain
    c.close()
    c = kgb.Context(0)
    c.generate(precision=kgb.MIXED, zones=(6, 6, 6), groups=32, quad=(4, 8), legendre=2)
    c.set_option("fused_ltimes", 1)
    c.set_option("fused_sweep", 1)
    assert c.get_option("fused_ltimes_active") == 0  # the LPlusTimes prologue takes the sweep
    c.close()
