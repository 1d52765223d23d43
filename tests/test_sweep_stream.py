"""The streamed FP32 sweep (sweep_stream.cu) against the per-step FP32 kernel and the oracle.

Both kernels evaluate the same diamond-difference recurrence (Kernel/SweepSubdomain.cpp:86-108)
with the same expressions, and the running faces cross tile boundaries through the plane arrays
unrounded, so psi, the planes and every iterate are bit for bit the same whatever the kernel and
the tile shape; the fused population partials are summed in the same order at the same tiles.
Shapes: 128 Gauss-Legendre directions (16 per octant set, 8 groups per 128-chain block),
direction sets of 8 (16 groups per block), 12 (8 groups, 96-chain blocks) and 24 (4 groups, 96
chains), partial tiles at the downwind ends, zone sets, group sets, a perturbed (non-uniform)
mesh, the reversed (adjoint) orientation, and 1 to 4 stages.
"""
import numpy as np
import pytest

from tests.test_gpu_parity import check, pair

pytestmark = pytest.mark.gpu

BASE = dict(zones=(9, 7, 10), quad=(8, 16), groups=16, legendre=2, scatter=1, geometry=1)


def sweep_with(ctx, rhs, xy, tz, stream, stages=2):
    ctx.set_option("sweep_stream", stream)
    ctx.set_option("sweep_stream_stages", stages)
    ctx.set_option("sweep_tile_xy", xy)
    ctx.set_option("sweep_tile_z", tz)
    ctx.upload("rhs", rhs)
    ctx.sweep_solver()
    assert ctx.get_option("sweep_stream_active") == stream
    return [ctx.download(n) for n in ("psi", "i_plane", "j_plane", "k_plane")]


@pytest.mark.parametrize("kw", [dict(), dict(zones=(10, 7, 10), zsets=(2, 1, 2)), dict(gset=2), dict(dset=16),
                                dict(perturb=1), dict(quad=(8, 12)), dict(quad=(8, 24), groups=12)])
def test_streamed_sweep_bitwise(oracle, kgb, kw):
    p, ctx = pair(oracle, kgb, precision=1, **dict(BASE, **kw))
    rhs = np.random.default_rng(11).uniform(0.0, 2.0, ctx.field_bytes("rhs") // 8)
    want = sweep_with(ctx, rhs, 44, 3, 0)
    for xy, tz, stages in [(44, 3, 2), (42, 1, 1), (44, 16, 3), (42, 5, 4), (42, 32, 2), (44, 7, 1)]:
        got = sweep_with(ctx, rhs, xy, tz, 1, stages)
        for g, w, n in zip(got, want, ("psi", "i_plane", "j_plane", "k_plane")):
            np.testing.assert_array_equal(g, w, err_msg="%s at %d/%d, %d stages" % (n, xy, tz, stages))
    p.set("rhs", rhs)
    p.sweep_solver()
    check(want[0], p.get("psi"), 1e-5)


def test_streamed_solve_populations_bitwise(oracle, kgb):
    """Solves (fused population partials, graph replay) with either kernel at the same tiles."""
    p, ctx = pair(oracle, kgb, precision=1, **BASE)
    runs = []
    for stream in (1, 0):
        ctx.set_option("sweep_stream", stream)
        ctx.set_option("sweep_tile_xy", 44)
        ctx.set_option("sweep_tile_z", 4)
        runs.append((ctx.solve(4), ctx.download("phi")))
    np.testing.assert_array_equal(runs[0][0], runs[1][0])
    np.testing.assert_array_equal(runs[0][1], runs[1][1])
    np.testing.assert_allclose(runs[0][0], p.solve(4), rtol=1e-5)


def test_streamed_block_jacobi_bitwise(oracle, kgb):
    """Block Jacobi sweeps every zone set in one launch from zeroed planes: same bits either kernel."""
    p, ctx = pair(oracle, kgb, precision=1, **dict(BASE, zones=(10, 8, 10), zsets=(2, 2, 1)))
    ctx.set_option("block_jacobi", 1)
    rhs = np.random.default_rng(13).uniform(0.0, 2.0, ctx.field_bytes("rhs") // 8)
    want = sweep_with(ctx, rhs, 44, 3, 0)
    got = sweep_with(ctx, rhs, 44, 3, 1)
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g, w)


def test_streamed_adjoint_bitwise(oracle, kgb):
    """The reversed orientation (the adjoint's transposed sweep) through unrolled gradients."""
    p, ctx = pair(oracle, kgb, precision=1, **dict(BASE, zones=(9, 8, 10), zsets=(1, 2, 1)))
    nx, ny, nz = 9, 8, 10
    det = np.zeros((nz, ny, nx))
    det[nz // 2:, ny // 2:, nx // 2:] = 1.0
    ctx.set_response(det.ravel())
    out = []
    for stream, xy in ((1, 42), (1, 44), (0, 44)):
        ctx.set_option("sweep_stream", stream)
        ctx.set_option("sweep_tile_xy", xy)
        ctx.set_option("sweep_tile_z", 3)
        out.append(ctx.gradient_unrolled(3))
    for o in out[1:]:
        assert o[0] == out[0][0] and o[3] == out[0][3]
        np.testing.assert_array_equal(o[1], out[0][1])
        np.testing.assert_array_equal(o[2], out[0][2])


def test_stream_applies_to_the_mixed_form_only(oracle, kgb):
    """FP64 keeps the per-step kernel (and its exact parity); shapes outside the streamed kernel's reach fall back."""
    p, ctx = pair(oracle, kgb, precision=0, **BASE)
    ctx.set_option("sweep_tile_xy", 42)
    assert ctx.get_option("sweep_stream") == 1 and ctx.get_option("sweep_stream_active") == 0
    rhs = np.random.default_rng(12).uniform(0.0, 1.0, ctx.field_bytes("rhs") // 8)
    p.set("rhs", rhs); ctx.upload("rhs", rhs)
    p.sweep_solver(); ctx.sweep_solver()
    check(ctx.download("psi"), p.get("psi"), 1e-12)
    ctx.close()
    # 6 directions per set (48 directions): no 16-byte direction runs
    p, ctx = pair(oracle, kgb, precision=1, **dict(BASE, quad=(4, 12)))
    ctx.set_option("sweep_tile_xy", 42)
    assert ctx.get_option("sweep_stream_active") == 0
    ctx.upload("rhs", rhs[:ctx.field_bytes("rhs") // 8])
    p.set("rhs", rhs[:ctx.field_bytes("rhs") // 8])
    p.sweep_solver(); ctx.sweep_solver()
    check(ctx.download("psi"), p.get("psi"), 1e-5)


def test_streamed_autotune_then_solve(oracle, kgb):
    p, ctx = pair(oracle, kgb, precision=1, **BASE)
    ctx.fill("psi", 0.0)
    ctx.iterate()
    tuned = ctx.autotune()
    assert tuned["sweep_tile_xy"] in (44, 42, 22)
    np.testing.assert_allclose(ctx.solve(3), p.solve(3), rtol=1e-5)
