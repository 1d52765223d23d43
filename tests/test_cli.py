"""The kripke command-line driver (kripke_gb300/bin/kripke).

CPU: flags are parsed and validated like the reference driver (usage on -h,
bad decompositions rejected before any GPU work).  GPU: the printed particle
counts of a solve equal the oracle's, and the figures of merit are reported.
"""
import json
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "kripke_gb300", "bin", "kripke")


@pytest.fixture(scope="module")
def cli():
    from kripke_gb300 import build
    build.build()
    assert os.path.exists(CLI)
    return CLI


def run(cli, *args, timeout=600):
    return subprocess.run([cli, *args], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=timeout)


def test_usage(cli):
    r = run(cli, "--help")
    assert r.returncode == 1
    assert "--quad [<ndirs>|<polar>:<azim>]" in r.stdout and "--layout <LAYOUT>" in r.stdout


@pytest.mark.parametrize("args,msg", [
    (["--groups", "5", "--gset", "2"], "evenly divided by number of groupsets"),
    (["--quad", "4", "--dset", "8"], "needs to be at least 8"),
    (["--arch", "Sequential"], "GB300 GPU path"),
    (["--procs", "2,1,1"], "one rank"),
    (["--niter", "0"], "at least one iteration"),
])
def test_rejects_bad_input(cli, args, msg):
    r = run(cli, *args)
    assert r.returncode != 0 and msg in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("extra,kw,rtol", [
    ([], dict(), 1e-12),
    (["--layout", "GZD", "--gset", "2", "--zset", "2,1,2"], dict(layout="GZD", gset=2, zsets=(2, 1, 2)), 1e-12),
    (["--precision", "mixed", "--autotune"], dict(), 1e-5),
    (["--pmethod", "bj", "--zset", "2,2,1"], dict(zsets=(2, 2, 1), block_jacobi=True), 1e-12),
])
def test_solve_matches_oracle(cli, oracle, extra, kw, rtol):
    base = ["--zones", "8,8,8", "--groups", "8", "--quad", "4:8", "--legendre", "2", "--niter", "4",
            "--geometry", "cube", "--scatter", "down", "--gset", "1", "--json"]
    args = base + extra
    r = run(cli, *args)
    assert r.returncode == 0, r.stdout[-3000:]
    printed = [float(x) for x in re.findall(r"iter \d+: particle count=([0-9.e+-]+)", r.stdout)]
    assert len(printed) == 4
    line = [l for l in r.stdout.splitlines() if l.startswith("{")][-1]
    fom = json.loads(line)
    assert fom["unknowns"] == 8 * 8 * 8 * 8 * 32 and fom["iterations"] == 4
    p = oracle.Problem(zones=(8, 8, 8), groups=8, quad=(4, 8), legendre=2, geometry=1, scatter=1,
                       **{"gset": 1, **kw})
    want = p.solve(4)
    # the solver prints the reference's %e (7 digits); the JSON line carries full precision
    np.testing.assert_allclose(printed, want, rtol=max(rtol, 5e-7))
    np.testing.assert_allclose(fom["particle_counts"], want, rtol=rtol)
    assert "Throughput:" in r.stdout and "TIMER_NAMES:" in r.stdout
