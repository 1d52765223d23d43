"""Captured solves: kgb_solve records the whole solve (psi reset and every
iteration with its particle count) into a CUDA graph once and replays it
while the context's tables are unchanged.  The replay must equal the
launch-by-launch solve bit for bit, and any change of inputs or options must
be picked up.
"""
import numpy as np
import pytest

KW = dict(zones=(10, 9, 8), groups=8, quad=(4, 8), legendre=2, geometry=1, scatter=1, gset=2, dset=8)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_graph_replay_equals_eager(kgb, precision):
    c = kgb.Context()
    c.generate(precision=precision, **KW)
    a = c.solve(6)
    assert c.get_option("graph_active") == 1
    psi_a = c.download("psi")
    b = c.solve(6)  # replay
    assert c.get_option("graph_active") == 1
    c.set_option("graph", 0)
    e = c.solve(6)
    assert c.get_option("graph_active") == 0
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(a, e)
    np.testing.assert_array_equal(psi_a, c.download("psi"))


@pytest.mark.gpu
def test_graph_follows_changes(kgb, oracle):
    c = kgb.Context()
    inp = c.generate(**KW)
    c.solve(4)
    # new tile shape: the captured solve must not be reused
    c.set_option("sweep_tile_xy", 22)
    c.set_option("sweep_tile_z", 2)
    got = c.solve(4)
    assert c.get_option("graph_active") == 1
    p = oracle.Problem(zones=KW["zones"], groups=8, quad=(4, 8), legendre=2, geometry=1, scatter=1, gset=2)
    np.testing.assert_allclose(got, p.solve(4), rtol=1e-12)
    # new cross sections (and with them the tabulated sweep reciprocals)
    st, sg = kgb.material_tables(inp)
    c.set_materials(st * 1.5, sg)
    p.set("sigt_zonal", p.get("sigt_zonal") * 1.5)
    np.testing.assert_allclose(c.solve(4), p.solve(4), rtol=1e-12)
    # another source strength is another graph
    a = np.array(c.solve(3, 2.0))
    b = np.array(c.solve(3, 1.0))
    np.testing.assert_allclose(a, 2.0 * b, rtol=1e-13)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_stream_split_is_bitwise_neutral(kgb, precision):
    # sweep steps launched in 1, 2 or 4 parts on separate streams (and the scattering's
    # launches alternating over two streams) compute the same values in the same order
    c = kgb.Context()
    c.generate(precision=precision, zsets=(2, 1, 1), **KW)
    out = []
    for n in (1, 2, 4):
        c.set_option("sweep_streams", n)
        assert c.get_option("sweep_streams") == n
        out.append((np.array(c.solve(4)), c.download("psi")))
    for parts, psi in out[1:]:
        np.testing.assert_array_equal(parts, out[0][0])
        np.testing.assert_array_equal(psi, out[0][1])
    with pytest.raises(kgb.KgbError):
        c.set_option("sweep_streams", 5)
