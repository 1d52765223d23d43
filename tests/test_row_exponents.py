"""Row exponents recorded by the producer of a tensor-core operand.

With "row_exponents" (FP64, tensor-core LTimes) the solver loop's sweep
records, for every (zone, group) row of psi, the largest biased exponent
(an atomic max over the lanes of each group), and the next LTimes scales its
digit split of the row by it instead of reading the row once more to find it;
that LTimes likewise records phi's exponents per (zone, moment) over the
groups for the tensor-core scattering's gathered rows.  A recorded value is
exactly what the consuming kernel would find, so every iterate is bit for bit
that of the option off.  Any other write of psi drops its record: the tests
below write psi in each of those ways -- with values far outside the swept
ones, so a stale record would overflow the digit split -- and check that the
next iteration still matches a context that never records.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KW = dict(zones=(10, 9, 8), groups=8, quad=(4, 8), legendre=3, geometry=1, scatter=1, gset=2, dset=8)


def pair(kgb, precision=None, **kw):
    out = []
    for on in (0, 1):
        c = kgb.Context()
        c.generate(precision=kgb.FP64 if precision is None else precision, **dict(KW, **kw))
        c.set_option("row_exponents", on)
        out.append(c)
    return out


def same(a, b, fields=("psi", "phi", "phi_out", "rhs")):
    for f in fields:
        np.testing.assert_array_equal(a.download(f), b.download(f), err_msg=f)


@pytest.mark.parametrize("kw", [dict(), dict(quad=(8, 16)), dict(quad=(8, 8)), dict(zsets=(2, 1, 2)),
                                dict(zsets=(5, 3, 1), block_jacobi=True), dict(groups=64, legendre=4),
                                dict(groups=12), dict(quad=(8, 12))])
def test_iterates_bitwise(kgb, kw):
    bj = kw.pop("block_jacobi", False)
    a, b = pair(kgb, **kw)
    for c in (a, b):
        c.set_option("block_jacobi", int(bj))
    pa = [a.iterate() for _ in range(4)]
    pb = [b.iterate() for _ in range(4)]
    assert b.get_option("psi_row_exponents_active") == 1 and a.get_option("psi_row_exponents_active") == 0
    assert b.get_option("psi_row_exponents_valid") == 1
    # phi's record needs a power-of-two run of group rows per zone
    assert b.get_option("phi_row_exponents_active") == int(kw.get("groups", 8) != 12)
    assert a.get_option("phi_row_exponents_active") == 0
    assert pa == pb
    same(a, b)
    # graph-replayed solves (psi = 0 first: its record is zeroed with it)
    np.testing.assert_array_equal(a.solve(5), b.solve(5))
    assert b.get_option("graph_active") == 1 and b.get_option("psi_row_exponents_valid") == 1
    same(a, b)
    np.testing.assert_array_equal(a.solve(5), b.solve(5))  # replay
    same(a, b)


@pytest.mark.parametrize("quad", [(4, 6), (4, 12)])
def test_unaligned_direction_sets_fall_back(kgb, quad):
    # 3 and 6 directions per set: a warp's groups share no aligned run of 4 lanes, nothing is recorded
    a, b = pair(kgb, quad=quad)
    assert [a.iterate() for _ in range(3)] == [b.iterate() for _ in range(3)]
    assert b.get_option("psi_row_exponents_active") == 0 and b.get_option("moments_tensor_ltimes") == 1
    same(a, b)


def test_record_over_two_k_chunks(kgb, oracle):
    # 192 directions (24 per set: runs of 8 lanes) take two tensor-core LTimes launches, each scaled
    # by the whole row's recorded exponent instead of its own chunk's: the same 54 bits of every
    # element relative to the row, so the iterates agree with the pass to FP64 rounding and with
    # the oracle to 1e-12
    kw = dict(zones=(6, 5, 7), groups=8, quad=(8, 24), legendre=3, geometry=1, scatter=1, gset=1, dset=8)
    a, b = pair(kgb, **kw)
    pa = [a.iterate() for _ in range(4)]
    pb = [b.iterate() for _ in range(4)]
    assert b.get_option("psi_row_exponents_active") == 1 and b.get_option("moments_tensor_ltimes") == 1
    np.testing.assert_allclose(pb, pa, rtol=1e-13)
    for f in ("psi", "phi"):
        got, want = b.download(f), a.download(f)
        assert np.max(np.abs(got - want)) <= 1e-13 * np.max(np.abs(want)), f
    p = oracle.Problem(**kw)
    np.testing.assert_allclose(b.solve(5), p.solve(5), rtol=1e-12)


def test_converged_solve_bitwise(kgb):
    a, b = pair(kgb)
    ra, rb = a.solve_converged(1.0, 1e-10, 200), b.solve_converged(1.0, 1e-10, 200)
    assert ra == rb
    same(a, b, ("psi", "phi"))


def _wild(shape, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(shape) * np.exp2(rng.integers(-40, 60, size=shape))


@pytest.mark.parametrize("how", ["upload", "fill", "sweep_subdomain", "sweep_solver", "adjoint", "ltimes_api"])
def test_other_psi_writes_drop_the_record(kgb, how):
    a, b = pair(kgb)
    for c in (a, b):
        c.iterate()
        c.iterate()
    assert b.get_option("psi_row_exponents_valid") == 1
    for c in (a, b):
        if how == "upload":
            c.upload("psi", _wild(c.download("psi").shape, 1))
        elif how == "fill":
            c.fill("psi", 3.0e80)
        elif how in ("sweep_subdomain", "sweep_solver"):
            c.upload("rhs", _wild(c.download("rhs").shape, 2))
            if how == "sweep_subdomain":
                c.sweep_subdomain(c.num_subdomains - 1)
            else:
                c.sweep_solver()
        elif how == "adjoint":
            # the adjoint state takes psi's place while it runs
            c.set_response(np.linspace(0.0, 1.0, 10 * 9 * 8))
            c.adjoint_solve(1e-8, 50)
        elif how == "ltimes_api":
            c.ltimes()  # reads psi only: the record stays
    if how == "ltimes_api":
        assert b.get_option("psi_row_exponents_valid") == 1
    else:
        assert b.get_option("psi_row_exponents_valid") == 0
    assert a.iterate() == b.iterate()
    same(a, b)
    assert a.iterate() == b.iterate()
    same(a, b)


def test_batched_solve_drops_the_record(kgb):
    bt = kgb.Batch(precision=kgb.FP64)
    bt.add(**KW)
    solo = kgb.Context()
    solo.generate(precision=kgb.FP64, **KW)
    solo.set_option("row_exponents", 0)
    c = bt.context(0)
    c.iterate()
    c.iterate()
    assert c.get_option("psi_row_exponents_valid") == 1
    bt.solve(3)  # writes the problem's psi through the batch's own kernels
    solo.solve(3)
    assert c.get_option("psi_row_exponents_valid") == 0
    np.testing.assert_array_equal(c.download("psi"), solo.download("psi"))
    assert c.iterate() == solo.iterate()
    np.testing.assert_array_equal(c.download("phi"), solo.download("phi"))


def test_zero_fill_records_zero_exponents(kgb):
    # kConst(psi, 0) before a solve: psi = 0 has row exponents 0, so the record stays usable
    a, b = pair(kgb)
    for c in (a, b):
        c.iterate()
        c.fill("psi", 0.0)
    assert b.get_option("psi_row_exponents_valid") == 1
    assert [a.iterate() for _ in range(3)] == [b.iterate() for _ in range(3)]
    same(a, b)


@pytest.mark.parametrize("kw", [dict(), dict(quad=(8, 16), legendre=4), dict(groups=64, legendre=4, zsets=(2, 1, 2)),
                                dict(groups=12)])
def test_mixed_form_phi_record_bitwise(kgb, kw):
    # the mixed form's register-tiled SIMT LTimes records phi's exponents for the tensor-core
    # scattering (the split-TF32 LTimes does not, and the zone-blocked FP32 scattering needs none:
    # both are turned off here)
    a, b = pair(kgb, precision=kgb.MIXED, **kw)
    for c in (a, b):
        c.set_option("moments_tf32", 0)
        c.set_option("scattering_block", 0)
        c.set_option("ltimes_symmetric", 0)  # the recording LTimes sums in ascending direction order
    pa = [a.iterate() for _ in range(4)]
    pb = [b.iterate() for _ in range(4)]
    assert b.get_option("phi_row_exponents_active") == int(kw.get("groups", 8) != 12)
    assert b.get_option("psi_row_exponents_active") == 0 and b.get_option("scattering_tensor_active") == 1
    assert pa == pb
    same(a, b)
    np.testing.assert_array_equal(a.solve(5), b.solve(5))
    same(a, b)
    ra, rb = a.solve_converged(1.0, 1e-5, 60), b.solve_converged(1.0, 1e-5, 60)
    assert ra == rb
    same(a, b, ("psi", "phi"))
