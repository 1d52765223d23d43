"""GPU parity: every hot-path kernel through the C ABI against the CPU oracle.

Inputs come from the oracle's generator (a restatement of Kripke's), are moved
across the ABI in Kripke's chunked host layout, and the outputs are compared
in the same layout.  Tolerances: the plain form is FP64 and must match to
1e-12 relative (fused multiply-adds and sum order are the only differences);
the mixed form is checked against the FP64 oracle at 1e-5 on single kernels
and 1e-6 norm-wise on phi after a solve.
"""
import numpy as np
import pytest

from tests.nesting import LAYOUTS

pytestmark = pytest.mark.gpu

INPUTS = ("ell", "ell_plus", "sigt_zonal", "data/sigs", "quadrature/xcos", "quadrature/ycos", "quadrature/zcos",
          "quadrature/w", "quadrature/id", "quadrature/jd", "quadrature/kd", "dx", "dy", "dz", "volume",
          "zone_to_num_mixelem", "zone_to_mixelem", "mixelem_to_zone", "mixelem_to_material",
          "mixelem_to_fraction", "moment_to_legendre")


def pair(oracle, kgb, precision=0, **kw):
    base = dict(zones=(6, 5, 7), groups=4, quad=16, legendre=2, gset=1, dset=8, niter=3)
    base.update(kw)
    p = oracle.Problem(**base)
    ctx = kgb.Context(0)
    ctx.setup_like(p.inp, precision=precision)
    for n in INPUTS:
        ctx.upload(n, p.get(n))
    return p, ctx


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def maxrel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def check(a, b, tol):
    assert rel(a, b) <= tol and maxrel(a, b) <= tol, (rel(a, b), maxrel(a, b))


@pytest.mark.parametrize("layout", LAYOUTS)
def test_field_roundtrip_all_layouts(oracle, kgb, layout):
    p, ctx = pair(oracle, kgb, layout=layout, gset=2, dset=16, zsets=(2, 1, 1), zones=(6, 5, 4))
    for n in INPUTS:
        np.testing.assert_array_equal(ctx.download(n), p.get(n), err_msg=n)
    rng = np.random.default_rng(1)
    for n in ("psi", "rhs", "phi", "phi_out", "i_plane", "j_plane", "k_plane", "sigt_zonal"):
        x = rng.standard_normal(ctx.field_bytes(n) // 8)
        ctx.upload(n, x)
        np.testing.assert_array_equal(ctx.download(n), x, err_msg=n)


@pytest.mark.parametrize("layout", ["DGZ", "ZGD", "GZD"])
def test_ltimes_lplustimes(oracle, kgb, layout):
    p, ctx = pair(oracle, kgb, layout=layout, quad=(4, 8), legendre=4, gset=2, dset=8, zones=(5, 4, 6))
    rng = np.random.default_rng(2)
    psi = rng.standard_normal(ctx.field_bytes("psi") // 8)
    p.set("psi", psi); ctx.upload("psi", psi)
    p.kconst("phi", 0.0); ctx.fill("phi", 0.0)
    p.ltimes(); ctx.ltimes()
    check(ctx.download("phi"), p.get("phi"), 1e-13)
    phi_out = rng.standard_normal(ctx.field_bytes("phi_out") // 8)
    p.set("phi_out", phi_out); ctx.upload("phi_out", phi_out)
    rhs0 = rng.standard_normal(ctx.field_bytes("rhs") // 8)
    p.set("rhs", rhs0); ctx.upload("rhs", rhs0)  # accumulate semantics
    p.lplustimes(); ctx.lplustimes()
    check(ctx.download("rhs"), p.get("rhs"), 1e-13)


@pytest.mark.parametrize("tensor", [1, 0])
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("quad", [(8, 16), (8, 24), (12, 24)])
def test_moment_transforms_wide_range(oracle, kgb, tensor, precision, quad):
    """LTimes / LPlusTimes on signed values spanning 30 decades, zero rows and partial tiles,
    through the tensor-core digit path (1) and the SIMT path (0); 192 and 288 directions run the
    tensor-core LTimes in several K chunks."""
    p, ctx = pair(oracle, kgb, precision=precision, quad=quad, legendre=4, zones=(7, 5, 3), groups=5)
    ctx.set_option("moments_tensor", tensor)
    rng = np.random.default_rng(11)
    n = ctx.field_bytes("psi") // 8
    psi = rng.standard_normal(n) * 10.0 ** rng.uniform(-30 if precision == 0 else -12, 3, n)
    psi[: n // 7] = 0.0
    p.set("psi", psi); ctx.upload("psi", psi)
    p.kconst("phi", 0.0); ctx.fill("phi", 0.0)
    p.ltimes(); ctx.ltimes()
    assert ctx.get_option("moments_tensor_ltimes") == tensor
    want, got = p.get("phi"), ctx.download("phi")
    tol = 1e-13 if precision == 0 else 2e-6
    scale = np.abs(want).max()
    assert np.max(np.abs(got - want)) <= tol * scale
    m = ctx.field_bytes("phi_out") // 8
    phi_out = rng.standard_normal(m) * 10.0 ** rng.uniform(-20 if precision == 0 else -8, 2, m)
    p.set("phi_out", phi_out); ctx.upload("phi_out", phi_out)
    p.kconst("rhs", 0.0); ctx.fill("rhs", 0.0)
    p.lplustimes(); ctx.lplustimes()
    assert ctx.get_option("moments_tensor_lplustimes") == tensor
    want, got = p.get("rhs"), ctx.download("rhs")
    assert np.max(np.abs(got - want)) <= tol * np.abs(want).max()


@pytest.mark.parametrize("quad", [(8, 16), (8, 24)])
def test_moment_transforms_many_tiles_per_sm(oracle, kgb, quad):
    """More 128-row tiles than SMs, so every CTA of the pipelined tensor-core kernel runs several
    tiles through its stages: 128 directions (two A stages) and 192 (one stage in FP64)."""
    p, ctx = pair(oracle, kgb, quad=quad, legendre=4, zones=(20, 20, 10), groups=8)
    ctx.set_option("moments_tensor", 1)
    rng = np.random.default_rng(13)
    psi = rng.standard_normal(ctx.field_bytes("psi") // 8)
    p.set("psi", psi); ctx.upload("psi", psi)
    p.kconst("phi", 0.0); ctx.fill("phi", 0.0)
    p.ltimes(); ctx.ltimes()
    check(ctx.download("phi"), p.get("phi"), 1e-13)
    phi_out = rng.standard_normal(ctx.field_bytes("phi_out") // 8)
    p.set("phi_out", phi_out); ctx.upload("phi_out", phi_out)
    p.kconst("rhs", 0.0); ctx.fill("rhs", 0.0)
    p.lplustimes(); ctx.lplustimes()
    assert ctx.get_option("moments_tensor_lplustimes") == 1
    check(ctx.download("rhs"), p.get("rhs"), 1e-13)


@pytest.mark.parametrize("scatter,gset", [(0, 1), (1, 1), (1, 4)])
@pytest.mark.parametrize("tensor", [1, 0])
def test_scattering_and_source(oracle, kgb, scatter, gset, tensor):
    """Scattering (accumulating into phi_out) and the source; tensor 1 puts the single-material
    zones on the tcgen05 digit products, tensor 0 keeps every zone on the SIMT kernel."""
    p, ctx = pair(oracle, kgb, scatter=scatter, gset=gset, groups=8, legendre=3, geometry=1, zones=(8, 6, 7))
    ctx.set_option("scattering_tensor", tensor)
    rng = np.random.default_rng(3)
    phi = rng.uniform(0.0, 1.0, ctx.field_bytes("phi") // 8)
    p.set("phi", phi); ctx.upload("phi", phi)
    out0 = rng.uniform(0.0, 1.0, ctx.field_bytes("phi_out") // 8)
    p.set("phi_out", out0); ctx.upload("phi_out", out0)
    p.scattering(); ctx.scattering()
    assert ctx.get_option("scattering_tensor_active") == tensor
    check(ctx.download("phi_out"), p.get("phi_out"), 1e-13)
    p.source(); ctx.source(1.0)
    check(ctx.download("phi_out"), p.get("phi_out"), 1e-13)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("groups,legendre", [(64, 4), (37, 2), (16, 0)])
def test_scattering_tensor_wide_range(oracle, kgb, precision, groups, legendre):
    """Tensor-core scattering on values spanning decades, zero moments and odd group counts,
    against the oracle (FP64 1e-13, mixed 2e-6 relative to the largest entry)."""
    p, ctx = pair(oracle, kgb, precision=precision, scatter=1, groups=groups, legendre=legendre, geometry=1,
                  zones=(9, 7, 5), quad=16)
    ctx.set_option("scattering_tensor", 1)
    ctx.set_option("scattering_block", 0)  # the mixed form's zone-blocked kernel is tested on its own
    rng = np.random.default_rng(5)
    n = ctx.field_bytes("phi") // 8
    phi = rng.standard_normal(n) * 10.0 ** rng.uniform(-20 if precision == 0 else -6, 2, n)
    phi[: n // 9] = 0.0
    p.set("phi", phi); ctx.upload("phi", phi)
    p.kconst("phi_out", 0.0); ctx.fill("phi_out", 0.0)
    p.scattering(); ctx.scattering()
    assert ctx.get_option("scattering_tensor_active") == 1
    want, got = p.get("phi_out"), ctx.download("phi_out")
    tol = 1e-13 if precision == 0 else 2e-6
    assert np.max(np.abs(got - want)) <= tol * np.abs(want).max()


@pytest.mark.parametrize("zones,zsets,dset,layout", [
    ((6, 5, 7), (1, 1, 1), 8, "DGZ"),
    ((9, 4, 5), (1, 1, 1), 16, "ZDG"),
    ((8, 6, 4), (2, 3, 2), 8, "GDZ"),
    ((13, 11, 9), (1, 1, 1), 8, "DZG"),
])
def test_sweep_solver(oracle, kgb, zones, zsets, dset, layout):
    p, ctx = pair(oracle, kgb, zones=zones, zsets=zsets, dset=dset, layout=layout, quad=(4, 8), groups=3)
    rng = np.random.default_rng(4)
    rhs = rng.uniform(0.0, 2.0, ctx.field_bytes("rhs") // 8)
    p.set("rhs", rhs); ctx.upload("rhs", rhs)
    p.sweep_solver(); ctx.sweep_solver()
    check(ctx.download("psi"), p.get("psi"), 1e-12)
    for n in ("i_plane", "j_plane", "k_plane"):
        check(ctx.download(n), p.get(n), 1e-12)


def test_sweep_subdomain_reads_incoming_planes(oracle, kgb):
    p, ctx = pair(oracle, kgb, zones=(5, 6, 7), quad=16, groups=2)
    rng = np.random.default_rng(5)
    for n in ("rhs", "i_plane", "j_plane", "k_plane"):
        x = rng.uniform(0.0, 1.0, ctx.field_bytes(n) // 8)
        p.set(n, x); ctx.upload(n, x)
    for s in (0, 3, 7):
        p.sweep_subdomain(s); ctx.sweep_subdomain(s)
    check(ctx.download("psi"), p.get("psi"), 1e-12)
    check(ctx.download("k_plane"), p.get("k_plane"), 1e-12)


@pytest.mark.parametrize("tz,txy", [(1, 44), (3, 44), (4, 42), (16, 22), (5, 42)])
def test_sweep_tile_shapes(oracle, kgb, tz, txy):
    p, ctx = pair(oracle, kgb, zones=(7, 9, 10), quad=16, groups=2)
    ctx.set_option("sweep_tile_z", tz)
    ctx.set_option("sweep_tile_xy", txy)
    rhs = np.random.default_rng(6).uniform(0.0, 1.0, ctx.field_bytes("rhs") // 8)
    p.set("rhs", rhs); ctx.upload("rhs", rhs)
    p.sweep_solver(); ctx.sweep_solver()
    check(ctx.download("psi"), p.get("psi"), 1e-12)


@pytest.mark.parametrize("recip", [0, 1])
def test_sweep_reciprocal_table_and_divide(oracle, kgb, recip):
    """Both denominator paths of the FP64 sweep (tabulated 1/den on a uniform mesh, or a divide per cell)."""
    p, ctx = pair(oracle, kgb, zones=(10, 9, 8), quad=(4, 8), groups=4, scatter=1, geometry=0, perturb=1)
    ctx.set_option("sweep_reciprocals", recip)
    want = p.solve(3)
    got = ctx.solve(3)
    np.testing.assert_allclose(got, want, rtol=1e-12)
    check(ctx.download("psi"), p.get("psi"), 1e-12)


@pytest.mark.parametrize("distinct,tabulated", [(40, 1), (60000, 1), (None, 0)])
def test_sweep_reciprocal_classes(oracle, kgb, distinct, tabulated):
    """The reciprocal table's sigt classes come from a device hash of the distinct
    values: a few dozen or 60000 distinct values are tabulated; with every one of the
    153600 values distinct (more than the 65535 classes, and more than the hash table
    holds) the sweep divides per cell; all sweep as the oracle does."""
    p, ctx = pair(oracle, kgb, zones=(48, 40, 40), quad=(4, 8), groups=2, scatter=1, geometry=1)
    n = ctx.field_bytes("sigt_zonal") // 8
    rng = np.random.default_rng(12)
    if distinct is None:
        sig = rng.permutation(np.linspace(0.05, 2.0, n))
    else:
        vals = rng.uniform(0.05, 2.0, distinct)
        sig = np.concatenate([vals, vals[rng.integers(0, distinct, n - distinct)]])
        rng.shuffle(sig)
    p.set("sigt_zonal", sig); ctx.upload("sigt_zonal", sig)
    rhs = rng.uniform(0.0, 1.0, ctx.field_bytes("rhs") // 8)
    p.set("rhs", rhs); ctx.upload("rhs", rhs)
    p.sweep_solver(); ctx.sweep_solver()
    assert ctx.get_option("sweep_reciprocals_active") == tabulated
    check(ctx.download("psi"), p.get("psi"), 1e-12)


def test_nonuniform_mesh(oracle, kgb):
    """Zone widths that vary along each axis (the sweep then divides per cell)."""
    p, ctx = pair(oracle, kgb, zones=(7, 6, 5), quad=16, groups=3, geometry=1)
    for n, k in (("dx", 7), ("dy", 6), ("dz", 5)):
        w = p.get(n) * (1.0 + 0.3 * np.sin(np.arange(k)))
        p.set(n, w); ctx.upload(n, w)
    rhs = np.random.default_rng(8).uniform(0.0, 1.0, ctx.field_bytes("rhs") // 8)
    p.set("rhs", rhs); ctx.upload("rhs", rhs)
    p.sweep_solver(); ctx.sweep_solver()
    check(ctx.download("psi"), p.get("psi"), 1e-12)


@pytest.mark.parametrize("precision", [0, 1])
def test_autotune_then_solve(oracle, kgb, precision):
    """The autotuner's choice keeps the sweep exact (FP64) / within the mixed tolerance."""
    p, ctx = pair(oracle, kgb, precision=precision, zones=(12, 10, 9), quad=(4, 8), groups=8, scatter=1, geometry=1)
    ctx.fill("psi", 0.0)
    ctx.iterate()
    tuned = ctx.autotune()
    assert tuned["sweep_tile_xy"] in (44, 42, 22) and tuned["sweep_ms"] > 0
    want = p.solve(3)
    got = ctx.solve(3)
    np.testing.assert_allclose(got, want, rtol=1e-12 if precision == 0 else 1e-5)


def test_population_and_balance(oracle, kgb):
    p, ctx = pair(oracle, kgb, scatter=1, quad=(4, 8), zones=(8, 8, 8), geometry=1)
    p.solve(2)
    ctx.solve(2)
    check(ctx.download("psi"), p.get("psi"), 1e-12)
    assert ctx.population() == pytest.approx(p.population(), rel=1e-12)
    gb, ob = ctx.balance(), p.balance()
    for k in range(4):
        assert gb[k] == pytest.approx(ob[k], rel=1e-12), k
    assert abs(gb[4]) <= 1e-11 * gb[0]


@pytest.mark.parametrize("quad", [96, (8, 12)])
def test_solve_config0(oracle, kgb, quad):
    """The 16^3 / 32-group / 96-direction / P4 / DGZ problem, 10 iterations."""
    p, ctx = pair(oracle, kgb, zones=(16, 16, 16), groups=32, quad=quad, legendre=4, gset=1, dset=8, geometry=1,
                  layout="DGZ")
    want = p.solve(10)
    got = ctx.solve(10)
    np.testing.assert_allclose(got, want, rtol=1e-12)
    ctx.fill("phi", 0.0); ctx.ltimes()
    p.kconst("phi", 0.0); p.ltimes()
    check(ctx.download("phi"), p.get("phi"), 1e-12)


@pytest.mark.parametrize("layout", LAYOUTS)
def test_solve_downscatter_all_layouts(oracle, kgb, layout):
    """Config-1 physics (GL quadrature, seeded downscatter) at a size the oracle finishes quickly."""
    p, ctx = pair(oracle, kgb, zones=(8, 8, 8), groups=16, quad=(4, 8), legendre=4, scatter=1, geometry=1,
                  layout=layout)
    want = p.solve(4)
    got = ctx.solve(4)
    np.testing.assert_allclose(got, want, rtol=1e-12)
    check(ctx.download("psi"), p.get("psi"), 1e-12)
    check(ctx.download("phi"), p.get("phi"), 1e-12)


def test_mixed_precision_phi_error(oracle, kgb):
    p, ctx = pair(oracle, kgb, precision=1, zones=(12, 12, 12), groups=16, quad=(4, 8), legendre=4, scatter=1,
                  geometry=1)
    want = p.solve(10)
    got = ctx.solve(10)
    np.testing.assert_allclose(got, want, rtol=1e-5)
    assert rel(ctx.download("phi"), p.get("phi")) <= 1e-6


@pytest.mark.parametrize("kw", [
    dict(zones=(16, 16, 16), groups=32, quad=96, legendre=4, geometry=1),
    dict(zones=(12, 10, 8), groups=16, quad=(8, 12), legendre=4, scatter=1, geometry=1, layout="GZD"),
    dict(zones=(8, 6, 10), groups=8, quad=(4, 8), legendre=3, scatter=1, perturb=1, geometry=0, gset=2,
         zsets=(2, 3, 1), layout="ZDG"),
    dict(zones=(6, 6, 6), groups=6, quad=32, legendre=2, perturb=1, dset=16, layout="DZG"),
])
def test_generator_matches_oracle(oracle, kgb, kw):
    """kgb_generate reproduces the oracle's restatement of Kripke's generator bit for bit."""
    p = oracle.Problem(**kw)
    ctx = kgb.Context(0)
    ctx.generate(**kw)
    for n in INPUTS:
        np.testing.assert_array_equal(ctx.download(n), p.get(n), err_msg=n)


def test_errors_are_reported(oracle, kgb):
    ctx = kgb.Context(0)
    with pytest.raises(kgb.KgbError) as e:
        ctx.ltimes()
    assert e.value.code == 6  # not set up
    ctx.setup(4, 4, 4, 2, 16, 1)
    with pytest.raises(kgb.KgbError) as e:
        ctx.ltimes()
    assert e.value.code == 6  # inputs missing
    with pytest.raises(kgb.KgbError) as e:
        ctx.upload("psi", np.zeros(3))
    assert e.value.code == 1
    with pytest.raises(kgb.KgbError) as e:
        ctx.upload("no_such_field", np.zeros(3))
    assert e.value.code == 1
    with pytest.raises(kgb.KgbError):
        ctx.setup(4, 4, 4, 3, 16, 1, gset=2)
