#!/usr/bin/env python
"""Golden vectors produced by the REFERENCE's own code.

LLNL Kripke's generator, Kernel::* functions, SweepSolver and SteadyStateSolver are compiled from
the reference sources by oracle/ref_build.sh (against the project-written stand-in for the RAJA
loop names, oracle/refshim/) and driven through oracle/pyref.py.  This script records what the
reference computes, so that tests can pin the oracle (and the GPU path) to the reference where
its sources are absent:

  tests/golden/ref_solves.json   per solve configuration: SHA-256 of every generated input field
                                 and of psi/phi/phi_out/rhs after SteadyStateSolver, the final
                                 population, and the reference CLI's printed particle counts
  tests/golden/ref_solves.npz    value samples of phi after each solve (for tolerance checks)
  tests/golden/ref_kernels.npz   seeded inputs and the reference's outputs of LTimes, LPlusTimes,
                                 scattering (dense lower-triangular sigs), source,
                                 sweepSubdomain (every subdomain, random incoming planes) and
                                 population on one small problem

Run where the reference sources are present (this writes nothing else):

    python tests/golden/make_ref_fixtures.py [reference-src-dir]
"""
import hashlib
import json
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle, pyref  # noqa: E402

# Solve configurations: the reference's own problem (Kobayashi 3i geometry, diagonal P0 sigs).
# "c0_*" are the CPU configuration's sizes (16^3 zones, 32 groups, 96 directions, P4, one group set,
# 8 direction sets, 10 iterations) with both of the reference's quadratures.
SOLVES = {
    "c0_s2": dict(zones=(16, 16, 16), groups=32, quad=96, legendre=4, gset=1, dset=8, niter=10),
    "c0_gl": dict(zones=(16, 16, 16), groups=32, quad=(8, 12), legendre=4, gset=1, dset=8, niter=10),
    "ref_default_dzg": dict(zones=(16, 16, 16), groups=32, quad=96, legendre=4, gset=2, dset=8, niter=4,
                            layout="DZG"),
    "gzd_sets": dict(zones=(6, 5, 7), groups=6, quad=(4, 6), legendre=3, gset=2, dset=8, niter=5, layout="GZD"),
    "zdg_zsets": dict(zones=(6, 6, 6), groups=4, quad=16, legendre=4, zsets=(2, 1, 2), niter=5, layout="ZDG"),
    "gdz_p0": dict(zones=(9, 4, 5), groups=3, quad=(4, 4), legendre=0, gset=3, dset=16, niter=5, layout="GDZ"),
    "zgd_p1_sub2": dict(zones=(5, 8, 4), groups=8, quad=32, legendre=1, gset=4, dset=8, zsets=(1, 2, 1), niter=5,
                        layout="ZGD", num_material_subsamples=2),
}
STATE = ("psi", "phi", "phi_out", "rhs")
# the reference CLI's printout on small problems (stdout "iter %d: particle count=%e, change=%e")
CLI_RUNS = {
    "cli_small": ["--zones", "8,8,8", "--groups", "8", "--quad", "32", "--niter", "5", "--legendre", "2"],
    "cli_gl_gzd": ["--zones", "6,8,5", "--groups", "4", "--quad", "4:8", "--niter", "4", "--legendre", "3",
                   "--layout", "GZD", "--gset", "2", "--zset", "1,2,1"],
}
KERNEL_INPUT = dict(zones=(4, 3, 5), groups=4, quad=16, legendre=3, gset=2, dset=8, layout="GZD")


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def phi_sample(p, kw):
    """phi values at 64 fixed positions per chunk plus the whole of its first 256 entries."""
    phi = p.get("phi")
    idx = np.unique(np.concatenate([np.arange(min(256, phi.size)),
                                    np.linspace(0, phi.size - 1, 2048).astype(np.int64)]))
    return idx, phi[idx]


def solves():
    out, samples = {}, {}
    for name, kw in SOLVES.items():
        r = pyref.Problem(**kw)
        rec = {"input": {k: (list(v) if isinstance(v, tuple) else v) for k, v in kw.items()},
               "fields": {n: digest(r.get(n)) for n in pyoracle.INPUT_NAMES}}
        rec["population"] = r.solve(kw["niter"])
        rec["state"] = {n: digest(r.get(n)) for n in STATE}
        idx, val = phi_sample(r, kw)
        samples[name + "/idx"], samples[name + "/phi"] = idx, val
        out[name] = rec
        r.close()
        print("reference solve", name, rec["population"], flush=True)
    for name, args in CLI_RUNS.items():
        res = subprocess.run([pyref.CLI_PATH, *args], stdout=subprocess.PIPE, text=True, check=True)
        counts = re.findall(r"iter \d+: particle count=([0-9.e+-]+)", res.stdout)
        out[name] = {"args": args, "particle_counts_printed": counts}
    return out, samples


def kernels():
    rng = np.random.default_rng(20261204)
    r = pyref.Problem(**KERNEL_INPUT)
    f = {}

    def put(name, arr):
        r.set(name, arr)
        return arr

    n_psi, n_phi = r.get("psi").size, r.get("phi").size
    # LTimes accumulates into phi
    f["ltimes/psi"] = put("psi", rng.standard_normal(n_psi))
    f["ltimes/phi0"] = put("phi", rng.standard_normal(n_phi))
    r.ltimes()
    f["ltimes/phi"] = r.get("phi")
    # LPlusTimes accumulates into rhs
    f["lplustimes/phi_out"] = put("phi_out", rng.standard_normal(n_phi))
    f["lplustimes/rhs0"] = put("rhs", rng.standard_normal(n_psi))
    r.lplustimes()
    f["lplustimes/rhs"] = r.get("rhs")
    # scattering with a dense lower-triangular transfer matrix per (material, order), then source
    G = KERNEL_INPUT["groups"]
    L1 = KERNEL_INPUT["legendre"] + 1
    sigs = np.zeros((3, L1, G, G))
    for m in range(3):
        for l in range(L1):
            sigs[m, l] = np.tril(rng.uniform(0.0, 1.0, (G, G))) / (2 * l + 1)
    f["scattering/sigs"] = put("data/sigs", sigs.ravel())
    f["scattering/phi"] = put("phi", rng.uniform(0.0, 1.0, n_phi))
    f["scattering/phi_out0"] = put("phi_out", rng.uniform(0.0, 1.0, n_phi))
    r.scattering()
    f["scattering/phi_out"] = r.get("phi_out")
    r.source()
    f["source/phi_out"] = r.get("phi_out")
    # sweepSubdomain of every subdomain from random rhs, sigt and incoming planes
    f["sweep/rhs"] = put("rhs", rng.uniform(0.0, 1.0, n_psi))
    f["sweep/sigt_zonal"] = put("sigt_zonal", rng.uniform(0.05, 2.0, r.get("sigt_zonal").size))
    for plane in ("i_plane", "j_plane", "k_plane"):
        f["sweep/%s0" % plane] = put(plane, rng.uniform(0.0, 1.0, r.get(plane).size))
    for s in range(r.num_sdoms):
        r.sweep_subdomain(s)
    f["sweep/psi"] = r.get("psi")
    for plane in ("i_plane", "j_plane", "k_plane"):
        f["sweep/%s" % plane] = r.get(plane)
    f["population/value"] = np.array([r.population()])
    r.close()
    return f


def main():
    if not pyref.available():
        if not pyref.build(sys.argv[1] if len(sys.argv) > 1 else None):
            sys.exit("the reference sources are not available: nothing written")
    rec, samples = solves()
    rec["_about"] = ("Outputs of LLNL Kripke's own code (compiled from its sources by oracle/ref_build.sh, "
                     "sequential policies, -O2 -ffp-contract=off on x86-64), written by "
                     "tests/golden/make_ref_fixtures.py")
    with open(os.path.join(HERE, "ref_solves.json"), "w") as fh:
        json.dump(rec, fh, indent=1, sort_keys=True)
    np.savez_compressed(os.path.join(HERE, "ref_solves.npz"), **samples)
    np.savez_compressed(os.path.join(HERE, "ref_kernels.npz"), input=json.dumps(KERNEL_INPUT), **kernels())
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
