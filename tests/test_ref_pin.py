"""The oracle pinned to the reference's own code.

Two records of what LLNL Kripke itself computes, both from its own C++ compiled from its sources
by oracle/ref_build.sh (sequential policies; RAJA's loop names supplied by oracle/refshim/):

- golden fixtures under tests/golden/ (written by tests/golden/make_ref_fixtures.py), which travel
  with the repository: the oracle reproduces them bit for bit -- every generated input field, the
  solved psi, phi, phi_out and rhs of the CPU configuration (16^3 zones, 32 groups, 96 directions,
  P4, 10 iterations; dummy S2 and Gauss-Legendre quadrature) and of smaller problems over every
  nesting with group, direction and zone sets, and single LTimes, LPlusTimes, scattering (dense
  lower-triangular transfer matrices), source and sweepSubdomain calls;
- the reference library itself (oracle/_ref/libkripke_ref.so) where it was built: the oracle
  agrees with it bit for bit on generated inputs, single kernels and whole solves over a wider
  matrix of configurations, including seeded downscatter and perturbed cross sections written into
  the reference's DataStore.

Populations are sums whose order differs (the reference's reducer against the oracle's fixed-order
sum; the threaded oracle's reduction), so they are held to 1e-14 relative (1e-12 for the threaded
sum over the 1.3e7 unknowns of the CPU configuration).
"""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import pyoracle, pyref

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
SOLVES = json.load(open(os.path.join(GOLDEN, "ref_solves.json")))
STATE = ("psi", "phi", "phi_out", "rhs")
THREADS = os.cpu_count() or 1


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def kwargs(rec):
    kw = {k: (tuple(v) if isinstance(v, list) else v) for k, v in rec["input"].items()}
    return kw


SOLVE_NAMES = sorted(k for k, v in SOLVES.items() if isinstance(v, dict) and "input" in v)


@pytest.mark.parametrize("name", SOLVE_NAMES)
def test_oracle_reproduces_reference_solves(oracle, name):
    """Generated inputs and the solved state equal the reference's bit for bit."""
    rec = SOLVES[name]
    kw = kwargs(rec)
    niter = kw.pop("niter")
    big = kw["zones"][0] * kw["zones"][1] * kw["zones"][2] * kw["groups"] > 50000
    # the OpenMP restatement forms psi and phi in the same per-element order as the sequential one
    p = oracle.Problem(threads=THREADS if big else 0, **kw)
    for n, want in rec["fields"].items():
        assert digest(p.get(n)) == want, "generated field %s differs from the reference's" % n
    part = p.solve(niter)
    for n, want in rec["state"].items():
        assert digest(p.get(n)) == want, "%s after %d iterations differs from the reference's" % (n, niter)
    # a sum of 10^7 terms in another order (the threaded reduction) differs by a few 1e-13
    assert abs(part[-1] - rec["population"]) <= (1e-12 if big else 1e-14) * abs(rec["population"])


def test_phi_samples_belong_to_the_solves():
    """The phi value samples (used by the GPU tests) are those of the recorded solves."""
    s = np.load(os.path.join(GOLDEN, "ref_solves.npz"))
    for name in SOLVE_NAMES:
        idx, val = s[name + "/idx"], s[name + "/phi"]
        assert idx.size == val.size > 256 and np.all(np.isfinite(val)) and np.abs(val).max() > 0


def _kernel_fixture():
    f = np.load(os.path.join(GOLDEN, "ref_kernels.npz"))
    kw = json.loads(str(f["input"]))
    kw["zones"] = tuple(kw["zones"])
    return f, kw


def run_kernel_sequence(p, f):
    """Drive a problem (oracle or reference) through the fixture's kernel calls; collect outputs."""
    out = {}
    p.set("psi", f["ltimes/psi"])
    p.set("phi", f["ltimes/phi0"])
    p.ltimes()
    out["ltimes/phi"] = p.get("phi")
    p.set("phi_out", f["lplustimes/phi_out"])
    p.set("rhs", f["lplustimes/rhs0"])
    p.lplustimes()
    out["lplustimes/rhs"] = p.get("rhs")
    p.set("data/sigs", f["scattering/sigs"])
    p.set("phi", f["scattering/phi"])
    p.set("phi_out", f["scattering/phi_out0"])
    p.scattering()
    out["scattering/phi_out"] = p.get("phi_out")
    p.source()
    out["source/phi_out"] = p.get("phi_out")
    p.set("rhs", f["sweep/rhs"])
    p.set("sigt_zonal", f["sweep/sigt_zonal"])
    for plane in ("i_plane", "j_plane", "k_plane"):
        p.set(plane, f["sweep/%s0" % plane])
    for s in range(p.num_sdoms):
        p.sweep_subdomain(s)
    out["sweep/psi"] = p.get("psi")
    for plane in ("i_plane", "j_plane", "k_plane"):
        out["sweep/%s" % plane] = p.get(plane)
    out["population/value"] = np.array([p.population()])
    return out


def test_oracle_reproduces_reference_kernels(oracle):
    f, kw = _kernel_fixture()
    got = run_kernel_sequence(oracle.Problem(**kw), f)
    for k, v in got.items():
        if k == "population/value":
            assert abs(v[0] - f[k][0]) <= 1e-14 * abs(f[k][0])
        else:
            np.testing.assert_array_equal(v, f[k], err_msg=k)


def test_reference_cli_printout_matches_oracle(oracle):
    """The reference driver's printed particle counts (%e) are the oracle's, rounded."""
    for name in ("cli_small", "cli_gl_gzd"):
        rec = SOLVES[name]
        a = rec["args"]
        opt = dict(zip(a[0::2], a[1::2]))
        quad = opt["--quad"]
        kw = dict(zones=tuple(int(x) for x in opt["--zones"].split(",")), groups=int(opt["--groups"]),
                  quad=tuple(int(x) for x in quad.split(":")) if ":" in quad else int(quad),
                  legendre=int(opt["--legendre"]))
        if "--layout" in opt:
            kw["layout"] = opt["--layout"]
        if "--gset" in opt:
            kw["gset"] = int(opt["--gset"])
        if "--zset" in opt:
            kw["zsets"] = tuple(int(x) for x in opt["--zset"].split(","))
        part = oracle.Problem(**kw).solve(int(opt["--niter"]))
        assert ["%e" % x for x in part] == rec["particle_counts_printed"], name


# ---- the live reference library (where the reference sources were present at build time) ------

live = pytest.mark.skipif(not pyref.available(), reason="oracle/_ref not built (no reference sources here)")

GEN_CASES = [
    dict(zones=(4, 4, 4), groups=2, quad=8, legendre=0),
    dict(zones=(7, 3, 5), groups=3, quad=48, legendre=5, layout="DZG", gset=3),
    dict(zones=(6, 6, 4), groups=4, quad=(4, 4), legendre=2, layout="GDZ", dset=16, zsets=(2, 3, 2)),
    dict(zones=(5, 5, 5), groups=8, quad=(8, 12), legendre=4, layout="ZGD", gset=2, num_material_subsamples=2),
    dict(zones=(10, 4, 6), groups=5, quad=(12, 6), legendre=3, layout="ZDG", gset=1, num_material_subsamples=1),
    dict(zones=(8, 8, 8), groups=6, quad=(4, 8), legendre=1, layout="GZD", gset=3, dset=8, zsets=(2, 2, 2),
         sigt=(0.3, 0.02, 0.7), sigs=(0.1, 0.01, 0.5), num_material_subsamples=8),
    dict(zones=(32, 8, 4), groups=2, quad=(16, 4), legendre=2, num_material_subsamples=2),
]


@live
@pytest.mark.parametrize("case", range(len(GEN_CASES)))
def test_live_generator_bit_for_bit(oracle, case):
    kw = GEN_CASES[case]
    p, r = oracle.Problem(**kw), pyref.Problem(**kw)
    for n in pyoracle.INPUT_NAMES:
        np.testing.assert_array_equal(p.get(n), r.get(n), err_msg=n)


@live
@pytest.mark.parametrize("layout", pyoracle.LAYOUTS)
def test_live_kernels_bit_for_bit(oracle, layout):
    kw = dict(zones=(5, 4, 3), groups=6, quad=(4, 4), legendre=4, gset=2, dset=16, zsets=(1, 2, 1), layout=layout)
    p, r = oracle.Problem(**kw), pyref.Problem(**kw)
    rng = np.random.default_rng(7)
    G, L1 = 6, 5
    sigs = np.zeros((3, L1, G, G))
    for m in range(3):
        for l in range(L1):
            sigs[m, l] = np.tril(rng.uniform(0.0, 1.0, (G, G))) / (2 * l + 1)
    f = {"ltimes/psi": rng.standard_normal(p.get("psi").size), "ltimes/phi0": rng.standard_normal(p.get("phi").size),
         "lplustimes/phi_out": rng.standard_normal(p.get("phi").size),
         "lplustimes/rhs0": rng.standard_normal(p.get("psi").size), "scattering/sigs": rng.uniform(0, 1, sigs.size),
         "scattering/phi": rng.uniform(0, 1, p.get("phi").size),
         "scattering/phi_out0": rng.uniform(0, 1, p.get("phi").size),
         "sweep/rhs": rng.uniform(0, 1, p.get("psi").size),
         "sweep/sigt_zonal": rng.uniform(0.05, 2.0, p.get("sigt_zonal").size)}
    for plane in ("i_plane", "j_plane", "k_plane"):
        f["sweep/%s0" % plane] = rng.uniform(0.0, 1.0, p.get(plane).size)
    a, b = run_kernel_sequence(p, f), run_kernel_sequence(r, f)
    for k in a:
        if k == "population/value":
            assert abs(a[k][0] - b[k][0]) <= 1e-14 * abs(b[k][0])
        else:
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@live
@pytest.mark.parametrize("scatter,perturb", [(1, 0), (0, 1), (1, 1)])
def test_live_solve_with_extended_cross_sections(oracle, scatter, perturb):
    """Seeded downscatter and perturbed cross sections (generator extensions the reference does not
    have) written into the reference's DataStore: the reference's kernels and solvers then give the
    oracle's solve bit for bit."""
    kw = dict(zones=(6, 4, 8), groups=8, quad=(4, 8), legendre=3, gset=2, dset=8, zsets=(1, 1, 2), layout="DZG")
    p = oracle.Problem(scatter=scatter, perturb=perturb, **kw)
    r = pyref.Problem(**kw)
    r.set("data/sigs", p.get("data/sigs"))
    r.set("sigt_zonal", p.get("sigt_zonal"))
    part = p.solve(6)
    pop = r.solve(6)
    for n in STATE:
        np.testing.assert_array_equal(p.get(n), r.get(n), err_msg=n)
    assert abs(part[-1] - pop) <= 1e-14 * abs(pop)
