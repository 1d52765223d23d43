"""Block Jacobi (--pmethod bj, src/Kripke/ParallelComm/BlockJacobiComm.cpp).

SweepSolver zeroes the planes (SweepSolver.cpp:28-30) before BlockJacobiComm
saves them and sends the saved copies downwind, so every subdomain is swept
from zero inflow on all faces and no subdomain waits on another.  The oracle
restates the comm object step by step; the CPU tests pin that restatement to
the property it implies, and the GPU tests compare the device path (one
launch over every subdomain) with it.
"""
import numpy as np
import pytest

KW = dict(zones=(8, 6, 5), groups=4, quad=(4, 8), legendre=2, geometry=1, scatter=1, gset=2, dset=8)


def random_rhs(p, seed=3):
    rhs = np.random.default_rng(seed).uniform(0.0, 2.0, p.get("rhs").size)
    p.set("rhs", rhs)
    return rhs


def test_bj_equals_independent_subdomain_sweeps(oracle):
    p = oracle.Problem(zsets=(2, 2, 1), block_jacobi=True, **KW)
    rhs = random_rhs(p)
    p.sweep_solver()
    bj = p.get("psi")
    q = oracle.Problem(zsets=(2, 2, 1), **KW)
    q.set("rhs", rhs)
    q.kconst("psi", 0.0)
    for s in range(q.num_sdoms):
        for n in ("i_plane", "j_plane", "k_plane"):
            q.kconst(n, 0.0)
        q.sweep_subdomain(s)
    np.testing.assert_array_equal(bj, q.get("psi"))


def test_bj_with_one_zone_set_is_the_sweep(oracle):
    a = oracle.Problem(block_jacobi=True, **KW)
    b = oracle.Problem(**KW)
    np.testing.assert_array_equal(a.solve(3), b.solve(3))
    np.testing.assert_array_equal(a.get("psi"), b.get("psi"))


def test_bj_decouples_zone_sets(oracle):
    # two zone sets in x: in every (group set, direction set) one of them has the
    # boundary upwind in x and sweeps exactly as in the sweep method; the other
    # loses the planes handed across the internal face
    a = oracle.Problem(zsets=(2, 1, 1), block_jacobi=True, **KW)
    b = oracle.Problem(zsets=(2, 1, 1), **KW)
    b.set("rhs", random_rhs(a))
    a.sweep_solver(); b.sweep_solver()
    n = a.num_sdoms
    ca, cb = np.split(a.get("psi"), n), np.split(b.get("psi"), n)
    same = [np.array_equal(x, y) for x, y in zip(ca, cb)]
    assert sum(same) == n // 2
    assert not np.allclose(a.solve(3), b.solve(3), rtol=1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("zsets,layout,precision", [((2, 2, 1), "DGZ", 0), ((1, 2, 5), "GZD", 0), ((2, 3, 1), "DGZ", 1)])
def test_bj_solve_matches_oracle(kgb, oracle, zsets, layout, precision):
    p = oracle.Problem(zsets=zsets, layout=layout, block_jacobi=True, **KW)
    want = p.solve(4)
    c = kgb.Context()
    c.generate(zsets=zsets, layout=layout, precision=precision, **KW)
    c.set_option("block_jacobi", 1)
    got = c.solve(4)
    tol = 1e-12 if precision == 0 else 1e-6
    np.testing.assert_allclose(got, want, rtol=tol)
    psi = c.download("psi")
    ref = p.get("psi")
    assert np.max(np.abs(psi - ref)) <= tol * np.abs(ref).max()


@pytest.mark.gpu
def test_bj_sweep_solver_and_graph_switch(kgb, oracle):
    p = oracle.Problem(zsets=(2, 1, 5), block_jacobi=True, **KW)
    c = kgb.Context()
    c.generate(zsets=(2, 1, 5), **KW)
    rhs = random_rhs(p)
    c.upload("rhs", rhs)
    c.set_option("block_jacobi", 1)
    assert c.get_option("block_jacobi") == 1
    p.sweep_solver(); c.sweep_solver()
    ref = p.get("psi")
    assert np.max(np.abs(c.download("psi") - ref)) <= 1e-12 * np.abs(ref).max()
    # a captured solve follows the method switch both ways
    bj = np.array(c.solve(3))
    c.set_option("block_jacobi", 0)
    sw = np.array(c.solve(3))
    q = oracle.Problem(zsets=(2, 1, 5), **KW)
    np.testing.assert_allclose(sw, q.solve(3), rtol=1e-12)
    c.set_option("block_jacobi", 1)
    np.testing.assert_array_equal(np.array(c.solve(3)), bj)
    with pytest.raises(kgb.KgbError):
        c.set_option("block_jacobi", 2)


@pytest.mark.gpu
def test_bj_gradient_matches_finite_differences(kgb):
    # the transpose of block Jacobi's block-diagonal sweep is the reversed sweep of
    # each subdomain from zero inflow: the adjoint solve runs it through the same switch
    # (the zone sets without source stay empty under block Jacobi, so the detector spans the mesh)
    from test_adjoint import BASE, fd_response, rel_err, solve_gradient
    ctx = kgb.Context()
    inp = ctx.generate(**dict(BASE, zsets=(2, 1, 2)))
    ctx.set_option("block_jacobi", 1)
    nz = int(np.prod(BASE["zones"]))
    ctx.set_response(np.linspace(0.5, 1.5, nz))
    st, sg = kgb.material_tables(inp)
    R, dt, ds, dq = solve_gradient(ctx)
    assert R > 0 and np.abs(dt).max() > 0 and np.abs(ds).max() > 0
    assert abs(R - dq) <= 1e-11 * abs(R)
    fd_t = np.zeros_like(dt)
    for m, g in zip(*np.unravel_index(np.argsort(-np.abs(dt), axis=None)[:3], dt.shape)):
        h = 1e-4 * st[m, g]
        s1, s2 = st.copy(), st.copy()
        s1[m, g] += h
        s2[m, g] -= h
        fd_t[m, g] = (fd_response(ctx, s1, sg) - fd_response(ctx, s2, sg)) / (2 * h)
        assert abs(dt[m, g] - fd_t[m, g]) <= 1e-6 * np.abs(dt).max(), (m, g, dt[m, g], fd_t[m, g])
    # the same problem under the sweep method has another fixed point and gradient
    ctx.set_materials(st, sg)
    ctx.set_option("block_jacobi", 0)
    R2, dt2, _, _ = solve_gradient(ctx)
    assert R2 > R and rel_err(dt2, dt) > 1e-3
