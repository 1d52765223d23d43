"""Fused sweep (mixed form): the solver loop forms rhs inside the sweep.

With "fused_sweep" the LPlusTimes launch of every iteration
(SteadyStateSolver.cpp:69-71) is dropped and the sweep forms each cell's rhs
from phi_out and ell_plus with the SIMT LPlusTimes kernel's arithmetic
(ascending moments, one FMA chain), so every iterate equals the unfused one
with the SIMT LPlusTimes bit for bit (the contexts here turn the split-TF32
tensor-core moments off).  rhs itself is refreshed lazily, as L+ phi_out, when
an entry point reads it.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KW = dict(zones=(12, 10, 9), groups=8, quad=(4, 8), legendre=4, geometry=1, scatter=1, gset=2, dset=8)


def pair(kgb, precision, **kw):
    out = []
    for fused in (0, 1):
        c = kgb.Context()
        c.generate(precision=precision, **dict(KW, **kw))
        c.set_option("moments_tf32", 0)
        c.set_option("fused_sweep", fused)
        out.append(c)
    return out


@pytest.mark.parametrize("kw", [dict(), dict(zsets=(2, 1, 3)), dict(zsets=(3, 2, 1), block_jacobi=True),
                                dict(legendre=2, layout="GZD")])
def test_fused_equals_unfused(kgb, kw):
    bj = kw.pop("block_jacobi", False)
    a, b = pair(kgb, kgb.MIXED, **kw)
    for c in (a, b):
        c.set_option("block_jacobi", int(bj))
    pa, pb = a.solve(5), b.solve(5)
    assert b.get_option("fused_sweep_active") == 1 and a.get_option("fused_sweep_active") == 0
    np.testing.assert_array_equal(pa, pb)
    np.testing.assert_array_equal(a.download("psi"), b.download("psi"))
    # rhs is formed again on demand and equals the one the unfused loop wrote
    np.testing.assert_array_equal(a.download("rhs"), b.download("rhs"))
    np.testing.assert_array_equal(np.array(a.balance()), np.array(b.balance()))
    # eager launches (no graph) take the same path
    b.set_option("graph", 0)
    np.testing.assert_array_equal(pa, b.solve(5))


def test_fused_then_kernel_api(kgb):
    a, b = pair(kgb, kgb.MIXED)
    a.solve(3)
    b.solve(3)
    # the Kernel API steps after a fused loop read the rhs that loop swept
    for c in (a, b):
        c.sweep_solver()
    np.testing.assert_array_equal(a.download("psi"), b.download("psi"))
    for c in (a, b):
        c.lplustimes()  # accumulates onto rhs = L+ phi_out
    np.testing.assert_array_equal(a.download("rhs"), b.download("rhs"))


def test_fused_adjoint_equals_unfused(kgb):
    a, b = pair(kgb, kgb.MIXED, zones=(8, 8, 8), legendre=2)
    grads = []
    for c in (a, b):
        c.set_response(np.linspace(0.0, 1.0, 8 * 8 * 8))
        c.solve_converged(1.0, -1.0, 30)
        c.adjoint_solve(-1.0, 30)
        grads.append(c.gradient())
    for x, y in zip(*grads):
        np.testing.assert_array_equal(np.asarray(x), np.asarray(y))


@pytest.mark.parametrize("precision,kw", [(0, dict()), (1, dict(legendre=5))])
def test_fused_inactive_outside_its_scope(kgb, precision, kw):
    # FP64 keeps the tensor-core LPlusTimes; the prologue holds at most 25 moments
    a, b = pair(kgb, precision, **kw)
    np.testing.assert_array_equal(a.solve(3), b.solve(3))
    assert b.get_option("fused_sweep") == 1 and b.get_option("fused_sweep_active") == 0
