"""Batched problems: one launch per kernel family, the sweeps of every problem
in one persistent launch (or each problem's own sweeps on parallel graph
branches), a solve replayed from a CUDA graph.

Parity: each problem's psi equals, bit for bit, that of the same problem's
own context run with the batch's sweep tiles (and the SIMT kernels when the
batch runs its batched SIMT kernels), since the arithmetic is term for term
the same; the particle counts agree to 1e-13 (the same sums in another order)
and match the CPU oracle within 1e-12 (FP64).
"""
import numpy as np
import pytest

from kripke_gb300.batching import uneven_inputs


def small_set(kgb, n=5, seed=11, precision=None):
    kw = dict(zones=(3, 10), groups=(2, 4, 8), directions=(32, 48, 64), legendre=(0, 2, 4))
    return uneven_inputs(n, seed=seed, precision=kgb.FP64 if precision is None else precision, **kw)


def make_batch(kgb, inputs, precision):
    b = kgb.Batch(precision=precision)
    for inp in inputs:
        b.add(inp)
    return b


def single_run(kgb, b, i, niter):
    c = b.context(i)
    c.set_option("sweep_tile_xy", b.get_option("sweep_tile_xy"))
    c.set_option("sweep_tile_z", b.get_option("sweep_tile_z"))
    if not b.get_option("per_problem_kernels"):
        c.set_option("moments_tf32", 0)
        c.set_option("moments_tensor", 0)
        c.set_option("scattering_tensor", 0)
        c.set_option("ltimes_symmetric", 0)  # the batched SIMT LTimes sums in ascending direction order
    return np.array(c.solve(niter)), c.download("psi")


def test_uneven_inputs_are_seeded(kgb):
    a = uneven_inputs(4, seed=5)
    b = uneven_inputs(4, seed=5)
    assert [(x.nx, x.ny, x.nz, x.num_groups, x.num_directions, x.seed) for x in a] == \
           [(x.nx, x.ny, x.nz, x.num_groups, x.num_directions, x.seed) for x in b]
    assert all(8 <= x.nx <= 48 and x.num_groups in (8, 16, 32, 64) and x.num_directions in (48, 96, 192) for x in a)


@pytest.mark.gpu
@pytest.mark.parametrize("prec,own", [("fp64", -1), ("fp64", 0), ("mixed", -1), ("mixed", 1)])
@pytest.mark.parametrize("tiles", [(22, 8), (44, 2), (42, 4)])
def test_batch_equals_single_contexts(kgb, prec, own, tiles):
    precision = kgb.FP64 if prec == "fp64" else kgb.MIXED
    b = make_batch(kgb, small_set(kgb, precision=precision), precision)
    b.set_option("sweep_tile_xy", tiles[0])
    b.set_option("sweep_tile_z", tiles[1])
    b.set_option("per_problem_kernels", own)
    niter = 4
    parts = b.solve(niter)
    assert b.get_option("graph_active") == 1
    psis = [b.context(i).download("psi") for i in range(len(b))]
    for i in range(len(b)):
        want, psi = single_run(kgb, b, i, niter)
        # a context's solve counts particles from each iteration's moments, the batch from its
        # fused sweep partials: the same sums in another order
        np.testing.assert_allclose(parts[:, i], want, rtol=1e-13)
        np.testing.assert_array_equal(psis[i], psi)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_batch_sweep_modes_agree(kgb, prec):
    """The persistent launch over all problems and each problem's own sweeps (the streamed FP32
    sweep where a problem's direction sets allow it: 16 and 24 directions per set here) give the
    same psi bit for bit; the particle counts are the same sums grouped by other blocks."""
    precision = kgb.FP64 if prec == "fp64" else kgb.MIXED
    inputs = uneven_inputs(5, seed=17, zones=(5, 12), groups=(8, 16), directions=(96, 128, 192), legendre=(2, 4),
                           precision=precision)
    b = make_batch(kgb, inputs, precision)
    runs = []
    for tiles in ((42, 4), (44, 8)):
        for mode in (0, 1):
            b.set_option("sweep_tile_xy", tiles[0])
            b.set_option("sweep_tile_z", tiles[1])
            b.set_option("per_problem_sweeps", mode)
            parts = b.solve(4)
            assert b.get_option("per_problem_sweeps") == mode and b.get_option("graph_active") == 1
            runs.append((parts, [b.context(i).download("psi") for i in range(len(b))]))
    for parts, psis in runs[1:]:
        np.testing.assert_allclose(parts, runs[0][0], rtol=1e-12)
        for got, want in zip(psis, runs[0][1]):
            np.testing.assert_array_equal(got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_batch_branches_agree(kgb, prec):
    """The branch count only spreads the problems' kernels over more or fewer streams: psi and the
    particle counts are the same bit for bit for 1, 4 and 8 branches; out-of-range counts are
    refused."""
    precision = kgb.FP64 if prec == "fp64" else kgb.MIXED
    inputs = uneven_inputs(6, seed=23, zones=(5, 10), groups=(8, 16), directions=(96, 128), legendre=(2, 4),
                           precision=precision)
    b = make_batch(kgb, inputs, precision)
    runs = []
    for nb in (4, 1, 8):
        b.set_option("branches", nb)
        assert b.get_option("branches") == nb
        parts = b.solve(3)
        runs.append((parts, [b.context(i).download("psi") for i in range(len(b))]))
    for parts, psis in runs[1:]:
        np.testing.assert_array_equal(parts, runs[0][0])
        for got, want in zip(psis, runs[0][1]):
            np.testing.assert_array_equal(got, want)
    for bad in (0, 9):
        with pytest.raises(Exception):
            b.set_option("branches", bad)


@pytest.mark.gpu
def test_batch_matches_oracle(kgb, oracle):
    inputs = small_set(kgb, n=4, seed=3)
    b = make_batch(kgb, inputs, kgb.FP64)
    parts = b.solve(5)
    for i, inp in enumerate(inputs):
        p = oracle.Problem(zones=(inp.nx, inp.ny, inp.nz), groups=inp.num_groups,
                           quad=(inp.quad_num_polar, inp.quad_num_azimuthal), legendre=inp.legendre_order, gset=1,
                           dset=8, geometry=1, scatter=1, sigt=tuple(inp.sigt), sigs=tuple(inp.sigs), seed=inp.seed)
        np.testing.assert_allclose(parts[:, i], p.solve(5), rtol=1e-12)


@pytest.mark.gpu
def test_batch_replay_is_deterministic(kgb):
    b = make_batch(kgb, small_set(kgb, n=6, seed=8), kgb.MIXED)
    a = b.solve(3)
    c = b.solve(3)
    np.testing.assert_array_equal(a, c)
    assert b.get_option("graph_active") == 1
    b.set_option("graph", 0)
    d = b.solve(3)
    assert b.get_option("graph_active") == 0
    np.testing.assert_array_equal(a, d)
    assert b.launch_count() == 3 * 3 * b.get_option("kernels_per_iteration")


@pytest.mark.gpu
def test_batch_autotune_then_parity(kgb):
    b = make_batch(kgb, small_set(kgb, n=4, seed=21), kgb.FP64)
    t = b.autotune()
    assert t["iteration_ms"] > 0 and t["sweep_tile_xy"] in (22, 42, 44) and t["sweep_tile_z"] in (2, 4, 8, 16)
    parts = b.solve(3)
    for i in range(len(b)):
        want, _ = single_run(kgb, b, i, 3)
        np.testing.assert_allclose(parts[:, i], want, rtol=1e-13)


@pytest.mark.gpu
def test_batch_rejects_unsupported(kgb):
    b = kgb.Batch(precision=kgb.FP64)
    with pytest.raises(kgb.KgbError):
        b.add(zones=(8, 8, 8), groups=4, quad=(4, 8), legendre=2, zsets=(2, 1, 1))
    with pytest.raises(kgb.KgbError):
        b.add(zones=(8, 8, 8), groups=4, quad=(4, 8), legendre=5)
    with pytest.raises(kgb.KgbError):
        b.solve(1)  # empty


@pytest.mark.gpu
def test_barrier_wait_gives_up_and_batch_recovers(kgb, oracle):
    """Failure path of the persistent sweep's grid barrier: with a wait limit of 0 ns every wait
    that finds the barrier still closed gives up at once, so the solve ends with KGB_ERR_TIMEOUT
    and a readable message (no trap, no hang; the waits record the failure and the launch runs
    to its end).  The batch stays usable: with the default limit restored, the next solve on the
    same problems matches the oracle."""
    inputs = small_set(kgb, n=4, seed=3)
    b = make_batch(kgb, inputs, kgb.FP64)
    assert b.get_option("barrier_wait_ns") == 2_000_000_000
    b.set_option("barrier_wait_ns", 0)
    with pytest.raises(kgb.KgbError) as err:
        b.solve(3)
    assert err.value.code == 4  # KGB_ERR_TIMEOUT
    assert "gave up" in str(err.value)
    b.set_option("barrier_wait_ns", 2_000_000_000)
    parts = b.solve(5)
    for i, inp in enumerate(inputs):
        p = oracle.Problem(zones=(inp.nx, inp.ny, inp.nz), groups=inp.num_groups,
                           quad=(inp.quad_num_polar, inp.quad_num_azimuthal), legendre=inp.legendre_order, gset=1,
                           dset=8, geometry=1, scatter=1, sigt=tuple(inp.sigt), sigs=tuple(inp.sigs), seed=inp.seed)
        np.testing.assert_allclose(parts[:, i], p.solve(5), rtol=1e-12)


@pytest.mark.gpu
def test_barrier_wait_option_is_checked(kgb):
    b = make_batch(kgb, small_set(kgb, n=2, seed=4), kgb.FP64)
    with pytest.raises(kgb.KgbError):
        b.set_option("barrier_wait_ns", -1)
    assert b.get_option("barrier_wait_ns") == 2_000_000_000
