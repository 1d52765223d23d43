"""The mixed form's TMA-fed SIMT LTimes (ltimes_stream.cu) against the register-tiled kernel.

Both form every output as the same FMA chain over ascending directions (Kernel/LTimes.cpp:54-65
restated with paired FP32 multiply-adds), so phi must agree bit for bit; the oracle bounds both.
Shapes: 96, 128 and 192 directions, Legendre orders 3 and 4 (16 and 25 moments), row counts that
leave a partial last 128-row tile, and 2 to 4 shared-memory stages.

Its octant-pair form (option ltimes_symmetric, on by default where L allows it) pairs each
direction of a 32-direction chunk's first 16 with its mirror image among the other 16 and sums
L(m, b) (psi(b) +- psi(b')): half the multiply-adds, another summation order, so it is held to
FP32 rounding against the bit-exact kernel and to the oracle; where L has no such pairs (96 and
192 directions) it must not be chosen.
"""
import numpy as np
import pytest

from tests.test_gpu_parity import check, pair

pytestmark = pytest.mark.gpu


def phi_after_ltimes(ctx, psi, stream, stages=2, sym=0):
    ctx.set_option("ltimes_stream", stream)
    ctx.set_option("ltimes_stream_stages", stages)
    ctx.set_option("ltimes_symmetric", sym)
    ctx.upload("psi", psi)
    ctx.iterate(want_population=False)  # phi = L psi first (the solver's LTimes, not accumulated)
    return ctx.download("phi")


@pytest.mark.parametrize("quad,legendre,zones,groups", [((8, 16), 4, (9, 7, 5), 8), ((8, 12), 3, (6, 5, 7), 12),
                                                        ((8, 24), 4, (5, 5, 3), 4)])
def test_streamed_ltimes_bitwise(oracle, kgb, quad, legendre, zones, groups):
    p, ctx = pair(oracle, kgb, precision=1, zones=zones, quad=quad, legendre=legendre, groups=groups, scatter=1,
                  geometry=1)
    psi = np.random.default_rng(31).uniform(-1.0, 2.0, ctx.field_bytes("psi") // 8)
    want = phi_after_ltimes(ctx, psi, 0)
    for stages in (2, 3, 4):
        got = phi_after_ltimes(ctx, psi, 1, stages)
        np.testing.assert_array_equal(got, want, err_msg="%d stages" % stages)
    p.set("psi", psi)
    p.kconst("phi", 0.0)
    p.ltimes()
    check(want, p.get("phi"), 1e-5)


@pytest.mark.parametrize("quad,legendre,zones,groups,active", [((8, 16), 4, (9, 7, 5), 8, 1),
                                                               ((8, 16), 3, (6, 5, 7), 12, 1),
                                                               ((4, 8), 4, (7, 6, 5), 16, 1),
                                                               ((8, 12), 4, (6, 5, 7), 8, 0),
                                                               ((8, 24), 4, (5, 5, 3), 4, 0)])
def test_octant_pair_ltimes(oracle, kgb, quad, legendre, zones, groups, active):
    p, ctx = pair(oracle, kgb, precision=1, zones=zones, quad=quad, legendre=legendre, groups=groups, scatter=1,
                  geometry=1)
    psi = np.random.default_rng(37).uniform(-1.0, 2.0, ctx.field_bytes("psi") // 8)
    exact = phi_after_ltimes(ctx, psi, 1)
    for stages in (2, 3):
        got = phi_after_ltimes(ctx, psi, 1, stages, sym=1)
        assert ctx.get_option("ltimes_symmetric_active") == active
        if active:
            # |d| <= 8 units of FP32 rounding of the largest output (sums of up to 192 terms of either sign)
            assert np.max(np.abs(got - exact)) <= 8 * 2.0 ** -24 * np.max(np.abs(exact)) * np.sqrt(quad[0] * quad[1])
        else:
            np.testing.assert_array_equal(got, exact)
    ctx.set_option("ltimes_symmetric", 1)
    p.set("psi", psi)
    p.kconst("phi", 0.0)
    p.ltimes()
    check(got, p.get("phi"), 1e-5)


def test_octant_pair_ltimes_in_the_adjoint(kgb):
    """The adjoint iteration runs LTimes with L+ in L's place (and L+'s own octant-pair table):
    unrolled gradients with the pairs on and off agree to FP32 rounding, and both to FP64."""
    kw = dict(zones=(6, 5, 4), groups=4, quad=(8, 16), legendre=4, geometry=1, scatter=1)
    out = {}
    for name, prec, sym in (("fp64", kgb.FP64, 0), ("pairs", kgb.MIXED, 1), ("ascending", kgb.MIXED, 0)):
        c = kgb.Context()
        c.generate(precision=prec, **kw)
        c.set_option("ltimes_symmetric", sym)
        c.set_response(np.linspace(0.0, 1.0, 6 * 5 * 4))
        out[name] = c.gradient_unrolled(6)
        if prec == kgb.MIXED:
            assert c.get_option("ltimes_symmetric_active") == sym
        c.close()
    for name, tol in (("ascending", 2e-6), ("fp64", 1e-5)):
        R, dt, ds, dq = out[name]
        Rp, dtp, dsp, dqp = out["pairs"]
        assert abs(Rp - R) <= tol * abs(R), name
        assert abs(dqp - dq) <= tol * abs(dq), name
        for a, b in ((dtp, dt), (dsp, ds)):
            assert np.max(np.abs(a - b)) <= tol * np.max(np.abs(b)), name
