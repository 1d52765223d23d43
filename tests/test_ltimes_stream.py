"""The mixed form's TMA-fed SIMT LTimes (ltimes_stream.cu) against the register-tiled kernel.

Both form every output as the same FMA chain over ascending directions (Kernel/LTimes.cpp:54-65
restated with paired FP32 multiply-adds), so phi must agree bit for bit; the oracle bounds both.
Shapes: 96, 128 and 192 directions, Legendre orders 3 and 4 (16 and 25 moments), row counts that
leave a partial last 128-row tile, and 2 to 4 shared-memory stages.
"""
import numpy as np
import pytest

from tests.test_gpu_parity import check, pair

pytestmark = pytest.mark.gpu


def phi_after_ltimes(ctx, psi, stream, stages=2):
    ctx.set_option("ltimes_stream", stream)
    ctx.set_option("ltimes_stream_stages", stages)
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
