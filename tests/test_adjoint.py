"""The adjoint of the source iteration and the response gradients.

CPU: the transposed-sweep identity the adjoint rests on, on the oracle's
reference sweep -- H^-T = V Rev V^-1, Rev the sweep from the opposite corner
and V the cell volumes -- for uniform and non-uniform meshes.
GPU: gradients from one adjoint solve against central finite differences of
the GPU forward solve and of the CPU oracle; the adjoint identity R = q dR/dq;
invariance under nesting, group sets and zone sets (which reverse the
zone-set wavefront and plane hand-off); non-uniform meshes; the mixed form.
Tolerances: FP64 gradients within 1e-6 of the finite differences (relative to
the largest component), the mixed form within 1e-5 of FP64.
"""
import numpy as np
import pytest

from nesting import logical_chunks

BASE = dict(zones=(6, 6, 6), groups=4, quad=(4, 8), legendre=2, geometry=1, scatter=1, perturb=1, gset=1)
TOL, MAXIT = 1e-14, 400


def detector(nx, ny, nz):
    det = np.zeros((nz, ny, nx))
    det[: nz // 2, :, nx // 2:] = 1.0
    det[nz - 1, ny - 1, 0] = 0.5
    return det.ravel()


# ---------------------------------------------------------------------------
# CPU: transposed sweep on the oracle
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("uniform", [True, False])
def test_transposed_sweep_identity(oracle, uniform):
    nx, ny, nz, G = 5, 4, 3, 2
    p = oracle.Problem(zones=(nx, ny, nz), groups=G, quad=(4, 8), legendre=0, gset=1, layout=0)
    rng = np.random.default_rng(7)
    if not uniform:
        for name, n in (("dx", nx), ("dy", ny), ("dz", nz)):
            p.set(name, rng.uniform(0.5, 2.0, n))
    dx, dy, dz = p.get("dx"), p.get("dy"), p.get("dz")
    vol = np.einsum("k,j,i->kji", dz, dy, dx).ravel()  # z = (k*ny + j)*nx + i
    n = p.get("psi").size
    V = np.tile(vol, n // vol.size)  # DGZ chunks [Ds][G][Z]: zone fastest

    def sweep(rhs):
        p.set("rhs", rhs)
        p.sweep_solver()
        return p.get("psi")

    a, b = rng.standard_normal(n), rng.standard_normal(n)
    Ta = sweep(a)
    for name in ("quadrature/id", "quadrature/jd", "quadrature/kd"):
        p.set(name, -p.get(name))
    TtB = V * sweep(b / V)
    lhs, rhs = float(b @ Ta), float(TtB @ a)
    assert abs(lhs - rhs) <= 1e-12 * (abs(lhs) + np.abs(b).sum() * np.abs(Ta).max())
    # a single reversed sweep is not the transpose on a non-uniform mesh without the volume scaling
    if not uniform:
        assert abs(float(sweep(b) @ a) - lhs) > 1e-6 * abs(lhs)


# ---------------------------------------------------------------------------
# GPU helpers
# ---------------------------------------------------------------------------
def make_ctx(kgb, precision=None, **kw):
    ctx = kgb.Context()
    args = dict(BASE, **kw)
    if precision is not None:
        args["precision"] = precision
    inp = ctx.generate(**args)
    nx, ny, nz = args["zones"]
    ctx.set_response(detector(nx, ny, nz))
    return ctx, inp


def solve_gradient(ctx, tol=TOL, to_floor=False):
    it, ch = ctx.solve_converged(1.0, tol, MAXIT)
    assert (ch <= tol or to_floor) and it < MAXIT
    ait, ach = ctx.adjoint_solve(tol, MAXIT)
    assert (ach <= tol or to_floor) and ait < MAXIT
    return ctx.gradient()


def fd_response(ctx, st, sg, q=1.0, tol=TOL):
    ctx.set_materials(st, sg)
    ctx.solve_converged(q, tol, MAXIT)
    return ctx.response()


def rel_err(got, want):
    got, want = np.asarray(got), np.asarray(want)
    return float(np.abs(got - want).max() / np.abs(want).max())


# ---------------------------------------------------------------------------
# GPU: gradients against finite differences of the GPU forward solve
# ---------------------------------------------------------------------------
@pytest.mark.gpu
def test_set_materials_reproduces_generator(kgb):
    ctx, inp = make_ctx(kgb)
    before = ctx.download("sigt_zonal"), ctx.download("data/sigs")
    st, sg = kgb.material_tables(inp)
    ctx.set_materials(st, sg)
    np.testing.assert_array_equal(ctx.download("sigt_zonal"), before[0])
    np.testing.assert_array_equal(ctx.download("data/sigs"), before[1])


@pytest.mark.gpu
def test_gradient_matches_gpu_finite_differences(kgb):
    ctx, inp = make_ctx(kgb)
    st, sg = kgb.material_tables(inp)
    R, dt, ds, dq = solve_gradient(ctx)
    assert R > 0
    G = inp.num_groups
    fd_t, fd_s = np.zeros((3, G)), np.zeros((3, G))
    for m in range(3):
        for g in range(G):
            h = 1e-4 * st[m, g]
            s1, s2 = st.copy(), st.copy()
            s1[m, g] += h
            s2[m, g] -= h
            fd_t[m, g] = (fd_response(ctx, s1, sg) - fd_response(ctx, s2, sg)) / (2 * h)
            h = 1e-4 * sg[m, 0, g, g]
            g1, g2 = sg.copy(), sg.copy()
            g1[m, 0, g, g] += h
            g2[m, 0, g, g] -= h
            fd_s[m, g] = (fd_response(ctx, st, g1) - fd_response(ctx, st, g2)) / (2 * h)
    ctx.set_materials(st, sg)
    fd_q = (fd_response(ctx, st, sg, 1.0 + 1e-3) - fd_response(ctx, st, sg, 1.0 - 1e-3)) / 2e-3
    assert rel_err(dt, fd_t) < 1e-6, (dt, fd_t)
    assert rel_err(ds, fd_s) < 1e-6, (ds, fd_s)
    assert abs(dq - fd_q) <= 1e-8 * abs(fd_q)


@pytest.mark.gpu
def test_adjoint_identity(kgb):
    # R is linear in the source strength, so R = q dR/dq = <lambda, b> at the fixed point
    ctx, _ = make_ctx(kgb)
    R, dt, ds, dq = solve_gradient(ctx)
    assert abs(R - dq) <= 1e-11 * abs(R)


@pytest.mark.gpu
def test_zero_detector_has_zero_gradient(kgb):
    ctx, inp = make_ctx(kgb)
    ctx.set_response(np.zeros(6 * 6 * 6))
    ctx.solve_converged(1.0, TOL, MAXIT)
    it, ch = ctx.adjoint_solve(TOL, MAXIT)
    assert it <= 2 and ch == 0.0
    R, dt, ds, dq = ctx.gradient()
    assert R == 0.0 and dq == 0.0 and not dt.any() and not ds.any()


@pytest.mark.gpu
def test_gradient_requires_adjoint(kgb):
    ctx, _ = make_ctx(kgb)
    ctx.solve_converged(1.0, 1e-8, MAXIT)
    with pytest.raises(kgb.KgbError):
        ctx.gradient()
    ctx.adjoint_solve(1e-8, MAXIT)
    ctx.gradient()
    ctx.set_response(None)  # a new response invalidates the adjoint state
    with pytest.raises(kgb.KgbError):
        ctx.gradient()


@pytest.mark.gpu
@pytest.mark.parametrize("kw", [
    dict(layout="GZD", gset=2),
    dict(zsets=(2, 3, 2), layout="ZDG"),
    dict(zsets=(3, 2, 1), gset=4, dset=16),
])
def test_gradient_independent_of_decomposition(kgb, kw):
    ref = solve_gradient(make_ctx(kgb)[0])
    got = solve_gradient(make_ctx(kgb, **kw)[0])
    assert abs(got[0] - ref[0]) <= 1e-12 * abs(ref[0])
    assert rel_err(got[1], ref[1]) < 1e-11
    assert rel_err(got[2], ref[2]) < 1e-11
    assert abs(got[3] - ref[3]) <= 1e-11 * abs(ref[3])


@pytest.mark.gpu
def test_gradient_nonuniform_mesh(kgb):
    ctx, inp = make_ctx(kgb, zsets=(2, 1, 3))
    rng = np.random.default_rng(3)
    d = {n: ctx.download(n) * rng.uniform(0.6, 1.4, ctx.download(n).size) for n in ("dx", "dy", "dz")}
    for n, v in d.items():
        ctx.upload(n, v)
    # volume per R chunk (zone sets 2 x 1 x 3 of 3 x 6 x 2 zones, Rz fastest), zone index (k*nys + j)*nxs + i
    vol = []
    for xs in range(2):
        for ys in range(1):
            for zs in range(3):
                vol.append(np.einsum("k,j,i->kji", d["dz"][2 * zs:2 * zs + 2], d["dy"], d["dx"][3 * xs:3 * xs + 3]).ravel())
    ctx.upload("volume", np.concatenate(vol))
    st, sg = kgb.material_tables(inp)
    R, dt, ds, dq = solve_gradient(ctx)
    assert abs(R - dq) <= 1e-11 * abs(R)
    for m, g in ((0, 0), (2, 3), (1, 1)):
        h = 1e-4 * st[m, g]
        s1, s2 = st.copy(), st.copy()
        s1[m, g] += h
        s2[m, g] -= h
        fd = (fd_response(ctx, s1, sg) - fd_response(ctx, s2, sg)) / (2 * h)
        assert abs(dt[m, g] - fd) <= 1e-6 * np.abs(dt).max(), (m, g, dt[m, g], fd)


@pytest.mark.gpu
def test_mixed_gradient_close_to_fp64(kgb):
    ref = solve_gradient(make_ctx(kgb)[0])
    ctx, _ = make_ctx(kgb, precision=kgb.MIXED)
    # FP32 iterates settle near 1e-7 relative change (the solves stop at that floor); measured errors
    # there are about 2e-6
    got = solve_gradient(ctx, tol=1e-9, to_floor=True)
    assert abs(got[0] - ref[0]) <= 1e-5 * abs(ref[0])
    assert rel_err(got[1], ref[1]) < 1e-5
    assert rel_err(got[2], ref[2]) < 1e-5
    assert abs(got[3] - ref[3]) <= 1e-5 * abs(ref[3])


# ---------------------------------------------------------------------------
# GPU gradients against finite differences of the CPU oracle
# ---------------------------------------------------------------------------
def oracle_response(p, det, G, L):
    """R of the oracle's current psi (layout DGZ, one group set, one zone set)."""
    info = p.sdom_info(0)
    Ds, Z = info["Ds"], info["nxs"] * info["nys"] * info["nzs"]
    nq = p.num_sdoms
    psi = np.concatenate(logical_chunks(p.get("psi"), "psi", "DGZ", (Ds, G, Z), nq))  # [D][G][Z]
    w = p.get("quadrature/w")
    vol = p.get("volume")
    sigt = p.get("sigt_zonal").reshape(G, Z)
    sigs = p.get("data/sigs").reshape(3, L + 1, G, G)
    colsum = sigs[:, 0].sum(axis=1)  # [m][g]: sum over destinations
    z2m, z2n = p.get("zone_to_mixelem"), p.get("zone_to_num_mixelem")
    mm, mf = p.get("mixelem_to_material"), p.get("mixelem_to_fraction")
    siga = sigt.copy()
    for z in range(Z):
        for e in range(z2m[z], z2m[z] + z2n[z]):
            siga[:, z] -= mf[e] * colsum[mm[e]]
    phiw = np.einsum("d,dgz->gz", w, psi)
    return float((det[None, :] * vol[None, :] * siga * phiw).sum())


def oracle_sigt_zonal(p, st):
    z2m, z2n = p.get("zone_to_mixelem"), p.get("zone_to_num_mixelem")
    mm, mf = p.get("mixelem_to_material"), p.get("mixelem_to_fraction")
    G, Z = st.shape[1], z2m.size
    out = np.zeros((G, Z))
    for z in range(Z):
        for e in range(z2m[z], z2m[z] + z2n[z]):
            out[:, z] += mf[e] * st[mm[e]]
    return out.ravel()


@pytest.mark.gpu
def test_gradient_matches_oracle_finite_differences(kgb, oracle):
    ctx, inp = make_ctx(kgb)
    R, dt, ds, dq = solve_gradient(ctx)
    G, L = inp.num_groups, inp.legendre_order
    st, sg = kgb.material_tables(inp)
    p = oracle.Problem(zones=BASE["zones"], groups=G, quad=BASE["quad"], legendre=L, geometry=1, scatter=1,
                       perturb=1, gset=1, layout=0)
    det = detector(*BASE["zones"])
    niter = 90

    def resp(st_, sg_):
        p.set("sigt_zonal", oracle_sigt_zonal(p, st_))
        p.set("data/sigs", sg_.ravel())
        p.solve(niter)
        return oracle_response(p, det, G, L)

    R_orc = resp(st, sg)
    assert abs(R - R_orc) <= 1e-11 * abs(R_orc)
    assert abs(dq - R_orc) <= 1e-10 * abs(R_orc)  # R is linear in q = 1
    fd_t, fd_s = np.zeros((3, G)), np.zeros((3, G))
    for m in range(3):
        for g in range(G):
            h = 1e-4 * st[m, g]
            s1, s2 = st.copy(), st.copy()
            s1[m, g] += h
            s2[m, g] -= h
            fd_t[m, g] = (resp(s1, sg) - resp(s2, sg)) / (2 * h)
            h = 1e-4 * sg[m, 0, g, g]
            g1, g2 = sg.copy(), sg.copy()
            g1[m, 0, g, g] += h
            g2[m, 0, g, g] -= h
            fd_s[m, g] = (resp(st, g1) - resp(st, g2)) / (2 * h)
    assert rel_err(dt, fd_t) < 1e-6, (dt, fd_t)
    assert rel_err(ds, fd_s) < 1e-6, (ds, fd_s)


@pytest.mark.gpu
def test_autograd_function(kgb):
    torch = pytest.importorskip("torch")
    from kripke_gb300.autograd import Problem
    pr = Problem(detector=detector(*BASE["zones"]), tol=TOL, max_iter=MAXIT, **BASE)
    st, ss, q = pr.parameters()
    R = pr.response(st, ss, q)
    (2.0 * R).backward()
    ref = solve_gradient(make_ctx(kgb)[0])
    assert abs(R.item() - ref[0]) <= 1e-12 * abs(ref[0])
    assert rel_err(st.grad.numpy(), 2 * ref[1]) < 1e-10
    assert rel_err(ss.grad.numpy(), 2 * ref[2]) < 1e-10
    assert abs(q.grad.item() - 2 * ref[3]) <= 1e-10 * abs(ref[3])
    # a second forward before backward: the backward restores its own state
    R1 = pr.response(st.detach().clone().requires_grad_(True), ss, q)
    pr.response(st.detach() * 1.1, ss.detach(), q.detach())
    R1.backward()
    assert torch.isfinite(R1)


# ---------------------------------------------------------------------------
# GPU: unrolled (checkpoint) mode -- gradients of the fixed-count solve
# ---------------------------------------------------------------------------
def unrolled_response(ctx, st, sg, niter, q=1.0):
    ctx.set_materials(st, sg)
    ctx.solve(niter, q)
    return ctx.response()


@pytest.mark.gpu
@pytest.mark.parametrize("niter,stride", [(1, 0), (5, 1), (7, 3), (10, 0), (6, 6)])
def test_unrolled_gradient_matches_finite_differences(kgb, niter, stride):
    ctx, inp = make_ctx(kgb)
    st, sg = kgb.material_tables(inp)
    R, dt, ds, dq = ctx.gradient_unrolled(niter, 1.0, stride)
    assert abs(R - unrolled_response(ctx, st, sg, niter)) <= 1e-13 * abs(R)
    assert abs(R - dq) <= 1e-11 * abs(R)  # R is linear in q after any iteration count
    for m, g in ((0, 0), (0, 3), (1, 2), (2, 1)):
        h = 1e-4 * st[m, g]
        s1, s2 = st.copy(), st.copy()
        s1[m, g] += h
        s2[m, g] -= h
        fd = (unrolled_response(ctx, s1, sg, niter) - unrolled_response(ctx, s2, sg, niter)) / (2 * h)
        assert abs(dt[m, g] - fd) <= 1e-6 * np.abs(dt).max(), (m, g, dt[m, g], fd)
        h = 1e-4 * sg[m, 0, g, g]
        g1, g2 = sg.copy(), sg.copy()
        g1[m, 0, g, g] += h
        g2[m, 0, g, g] -= h
        fd = (unrolled_response(ctx, st, g1, niter) - unrolled_response(ctx, st, g2, niter)) / (2 * h)
        assert abs(ds[m, g] - fd) <= 1e-6 * np.abs(ds).max(), (m, g, ds[m, g], fd)


@pytest.mark.gpu
def test_unrolled_stride_independent_and_converges(kgb):
    ctx, _ = make_ctx(kgb)
    a = ctx.gradient_unrolled(9, 1.0, 1)
    b = ctx.gradient_unrolled(9, 1.0, 4)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)  # recomputed iterates are bitwise the stored ones
    ref = solve_gradient(ctx)
    long = ctx.gradient_unrolled(120, 1.0, 0)
    assert abs(long[0] - ref[0]) <= 1e-12 * abs(ref[0])
    assert rel_err(long[1], ref[1]) < 1e-10
    assert rel_err(long[2], ref[2]) < 1e-10
