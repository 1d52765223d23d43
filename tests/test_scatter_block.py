"""Zone-blocked FP32 scattering of the mixed form (scatter.cu, scatter_block_kernel).

The kernel stages a material's transfer matrices and a run of its single-material zones in shared
memory and sums, for every (zone, destination group), the same terms in the same order as the SIMT
scattering kernel (source groups ascending; exact zeros outside a row's nonzero range), so its
outputs must equal that kernel's bit for bit: single calls (accumulating onto phi_out, as
Kernel::scattering does, Kernel/Scattering.cpp:79-98), whole solves and adjoint gradients, over
group counts that fill a warp, pack several zones into one, or leave lanes idle, and odd group
counts whose matrices end off a 16-byte boundary of shared memory.  Against the FP64
oracle the outputs stay within FP32 rounding.
"""
import numpy as np
import pytest

from tests.test_gpu_parity import pair

pytestmark = pytest.mark.gpu


def scatter_both(ctx, phi, out0):
    res = []
    for block in (1, 0):
        ctx.set_option("scattering_block", block)
        ctx.upload("phi", phi)
        ctx.upload("phi_out", out0)
        ctx.scattering()
        res.append((ctx.get_option("scattering_block_active"), ctx.download("phi_out")))
    ctx.set_option("scattering_block", 1)
    return res


@pytest.mark.parametrize("groups,legendre", [(64, 4), (32, 2), (16, 3), (8, 4), (12, 1), (48, 0), (64, 1), (37, 2), (5, 3), (63, 4), (1, 1)])
def test_block_scattering_bitwise(oracle, kgb, groups, legendre):
    p, ctx = pair(oracle, kgb, precision=kgb.MIXED, groups=groups, legendre=legendre, zones=(10, 9, 8), quad=(4, 8),
                  scatter=1, geometry=1)
    ctx.set_option("scattering_tensor", 0)
    rng = np.random.default_rng(groups * 10 + legendre)
    n = ctx.field_bytes("phi") // 8
    phi = rng.uniform(-1.0, 1.0, n).astype(np.float32).astype(np.float64)
    out0 = rng.uniform(0.0, 1.0, n).astype(np.float32).astype(np.float64)
    (on, blk), (off, simt) = scatter_both(ctx, phi, out0)
    assert on == 1 and off == 0
    np.testing.assert_array_equal(blk, simt)
    p.set("phi", phi)
    p.set("phi_out", out0)
    p.scattering()
    want = p.get("phi_out")
    assert np.max(np.abs(blk - want)) <= 2e-6 * np.max(np.abs(want))
    ctx.close()


@pytest.mark.parametrize("kw", [dict(), dict(gset=2, layout="GZD", zsets=(2, 1, 1)), dict(groups=16, legendre=2)])
def test_block_scattering_solve_and_adjoint_bitwise(kgb, kw):
    base = dict(zones=(8, 8, 8), groups=32, quad=(4, 8), legendre=4, geometry=1, scatter=1)
    base.update(kw)
    out = []
    for block in (1, 0):
        c = kgb.Context(0)
        c.generate(precision=kgb.MIXED, **base)
        c.set_option("scattering_tensor", 0)
        c.set_option("scattering_block", block)
        parts = c.solve(6)
        psi = c.download("psi")
        c.set_response(np.linspace(0.0, 1.0, 8 * 8 * 8))
        c.solve_converged(1.0, -1.0, 20)
        c.adjoint_solve(-1.0, 20)
        grad = c.gradient()
        out.append((c.get_option("scattering_block_active"), parts, psi, grad))
        c.close()
    (on, pa, sa, ga), (off, pb, sb, gb) = out
    assert on == 1 and off == 0
    np.testing.assert_array_equal(pa, pb)
    np.testing.assert_array_equal(sa, sb)
    for x, y in zip(ga, gb):
        np.testing.assert_array_equal(np.asarray(x), np.asarray(y))


@pytest.mark.parametrize("groups,legendre,zones", [(64, 4, (32, 32, 16)), (16, 2, (24, 20, 16)), (4, 1, (40, 16, 12)),
                                                    (48, 3, (16, 16, 20))])
def test_staged_block_scattering_many_items(kgb, groups, legendre, zones):
    """Enough zones that each 128-thread group of the staged kernel (groups a multiple of 4) runs
    many items of every material, the next item's copies in flight while the last one is stored."""
    ctx = kgb.Context(0)
    ctx.generate(precision=kgb.MIXED, groups=groups, legendre=legendre, zones=zones, quad=(4, 8), scatter=1,
                 geometry=1)
    ctx.set_option("scattering_tensor", 0)
    rng = np.random.default_rng(groups + 100 * legendre)
    n = ctx.field_bytes("phi") // 8
    phi = rng.uniform(-1.0, 1.0, n).astype(np.float32).astype(np.float64)
    out0 = rng.uniform(0.0, 1.0, n).astype(np.float32).astype(np.float64)
    (on, blk), (off, simt) = scatter_both(ctx, phi, out0)
    assert on == 1 and off == 0
    np.testing.assert_array_equal(blk, simt)
    ctx.close()


def test_block_scattering_not_in_fp64(oracle, kgb):
    p, ctx = pair(oracle, kgb, precision=kgb.FP64, groups=8, legendre=2)
    assert ctx.get_option("scattering_block_active") == 0
    ctx.close()
