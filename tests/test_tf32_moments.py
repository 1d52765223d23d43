"""The mixed form's LTimes and LPlusTimes as split-TF32 tensor-core GEMMs (tf32_moments.cu).

Each FP32 element of A is split exactly into three TF32 pieces (truncation), B likewise on the
host (rounding), and every product taken as the six terms up to 2^-20 of the leading one, the
small terms first, the leading ones last, with FP32 accumulation in tensor memory.  Checked
through the C ABI against the FP64 oracle (whose kernels equal the reference's bit for bit):
elementwise within 8 * 2^-22 * sum_k |a_k b_k| + 2^-20 * |C| of the FP64 result, and with a
largest error at most twice that of the FP32 SIMT kernel on the same inputs -- on tail tiles,
several tiles per CTA, every supported width, and in the accumulating form of the kernel entry
points (bulk reduce-adds).  Whole mixed solves with the TF32 kernels stay within the mixed form's
1e-6 of the FP64 oracle (2-norm ratio).

The tensor core's accumulation truncates, so each accumulation at a sum's full magnitude pulls it
towards zero by up to one unit in the last place, and over a source iteration with strong
scattering that bias adds up where the SIMT kernels' round-to-nearest errors cancel.  LPlusTimes
adds its leading products in descending moment order (moment 0, which dominates, last), which
brings it to the SIMT kernel's error; LTimes has no dominant direction, so its TF32 kernel is
opt-in ("moments_tf32_ltimes") and the mixed default keeps the SIMT LTimes.
"""
import numpy as np
import pytest

from tests.test_gpu_parity import pair

pytestmark = pytest.mark.gpu


def bound(a_abs_dot, want):
    return 8 * 2.0 ** -22 * a_abs_dot + 2.0 ** -20 * np.abs(want)


def run_both(ctx, op, fill):
    """op through the TF32 kernel, then through the FP32 SIMT kernel, from the same inputs."""
    out = []
    for tf32 in (1, 0):
        ctx.set_option("moments_tf32", tf32)
        ctx.set_option("moments_tf32_ltimes", tf32)
        fill()
        op()
        out.append(ctx.get_option("moments_tf32_ltimes" if op == ctx.ltimes else "moments_tf32_lplustimes"))
        out.append(ctx.download("phi" if op == ctx.ltimes else "rhs"))
    ctx.set_option("moments_tf32", 1)
    return out


@pytest.mark.parametrize("quad,legendre,zones,groups", [
    ((8, 16), 4, (7, 5, 3), 5),      # 525 rows: a partial last tile
    ((8, 16), 4, (24, 24, 16), 8),   # 73,728 rows: several tiles per CTA
    ((4, 12), 2, (6, 6, 6), 8),      # 48 directions: the last K chunk half empty; 9 moments (N = 16)
    ((8, 24), 3, (9, 7, 5), 6),      # 192 directions, 16 moments
    ((8, 32), 4, (5, 5, 4), 4),      # 256 directions
    # one accumulator per tile and more K chunks than A slots, several tiles per CTA
    ((8, 24), 4, (24, 24, 16), 8),   # LTimes: 6 chunks, 3 slots; LPlusTimes: N = 192
    ((8, 32), 4, (24, 24, 12), 8),   # LTimes: 8 chunks, 2 slots; LPlusTimes: N = 256
])
def test_tf32_ltimes_lplustimes(oracle, kgb, quad, legendre, zones, groups):
    p, ctx = pair(oracle, kgb, precision=kgb.MIXED, quad=quad, legendre=legendre, zones=zones, groups=groups)
    assert ctx.get_option("moments_tf32") == 1
    rng = np.random.default_rng(5)
    n = ctx.field_bytes("psi") // 8
    psi = rng.standard_normal(n) * 10.0 ** rng.uniform(-3, 3, n)
    psi = psi.astype(np.float32).astype(np.float64)
    phi0 = rng.standard_normal(ctx.field_bytes("phi") // 8).astype(np.float32).astype(np.float64)
    # LTimes accumulates: phi0 + L psi
    p.set("psi", psi)
    p.set("phi", np.zeros_like(phi0))
    p.ltimes()
    want = p.get("phi") + phi0
    ctx.upload("psi", psi)
    on, got, off, simt = run_both(ctx, ctx.ltimes, lambda: ctx.upload("phi", phi0))
    assert on == 1 and off == 0
    p.set("psi", np.abs(psi)); p.set("phi", np.zeros_like(phi0))
    ell = p.get("ell"); p.set("ell", np.abs(ell)); p.ltimes(); absdot = p.get("phi"); p.set("ell", ell)
    assert np.all(np.abs(got - want) <= bound(absdot, want) + 2.0 ** -23 * np.abs(phi0))
    e_tf, e_simt = np.max(np.abs(got - want)), np.max(np.abs(simt - want))
    print("LTimes D=%d M=%d: max error TF32 %.3e, SIMT %.3e (of max %.3e)" %
          (quad[0] * quad[1], (legendre + 1) ** 2, e_tf, e_simt, np.max(np.abs(want))))
    assert e_tf <= 2.0 * e_simt + 2.0 ** -24 * np.max(np.abs(want))
    # LPlusTimes accumulates: rhs0 + L+ phi_out
    m = ctx.field_bytes("phi_out") // 8
    phi_out = (rng.standard_normal(m) * 10.0 ** rng.uniform(-3, 3, m)).astype(np.float32).astype(np.float64)
    rhs0 = rng.standard_normal(n).astype(np.float32).astype(np.float64)
    p.set("phi_out", phi_out)
    p.set("rhs", np.zeros_like(rhs0))
    p.lplustimes()
    want = p.get("rhs") + rhs0
    ctx.upload("phi_out", phi_out)
    on, got, off, simt = run_both(ctx, ctx.lplustimes, lambda: ctx.upload("rhs", rhs0))
    D = quad[0] * quad[1]
    assert on == (1 if D <= 256 and D % 16 == 0 else 0) and off == 0
    p.set("phi_out", np.abs(phi_out)); p.set("rhs", np.zeros_like(rhs0))
    ellp = p.get("ell_plus"); p.set("ell_plus", np.abs(ellp)); p.lplustimes(); absdot = p.get("rhs")
    assert np.all(np.abs(got - want) <= bound(absdot, want) + 2.0 ** -23 * np.abs(rhs0))
    e_tf, e_simt = np.max(np.abs(got - want)), np.max(np.abs(simt - want))
    print("LPlusTimes D=%d M=%d: max error TF32 %.3e, SIMT %.3e (of max %.3e)" %
          (D, (legendre + 1) ** 2, e_tf, e_simt, np.max(np.abs(want))))
    assert e_tf <= 2.0 * e_simt + 2.0 ** -24 * np.max(np.abs(want))
    ctx.close()


@pytest.mark.parametrize("kw", [
    dict(zones=(12, 10, 8), groups=8, quad=(8, 16), legendre=4, geometry=1, scatter=1),
    dict(zones=(8, 8, 8), groups=16, quad=(4, 12), legendre=2, gset=2, dset=8, zsets=(2, 1, 1), layout="ZGD",
         geometry=1, scatter=1),
])
def test_tf32_solve_against_fp64(oracle, kgb, kw):
    """A mixed solve with the TF32 kernels in its loop against the FP64 oracle, and against the same
    mixed solve with the FP32 SIMT kernels."""
    p, ctx = pair(oracle, kgb, precision=kgb.MIXED, **kw)
    ctx.set_option("moments_tf32_ltimes", 1)
    want_parts = p.solve(8)
    parts = ctx.solve(8)
    assert ctx.get_option("moments_tf32_ltimes") == 1 and ctx.get_option("moments_tf32_lplustimes") == 1
    want, got = p.get("phi"), ctx.download("phi")
    ctx.set_option("moments_tf32", 0)
    ctx.solve(8)
    assert ctx.get_option("moments_tf32_ltimes") == 0
    simt = ctx.download("phi")
    e_tf = np.linalg.norm(got - want) / np.linalg.norm(want)
    e_simt = np.linalg.norm(simt - want) / np.linalg.norm(want)
    m_tf = np.max(np.abs(got - want)) / np.max(np.abs(want))
    m_simt = np.max(np.abs(simt - want)) / np.max(np.abs(want))
    print("solve: phi error (2-norm / max-abs) TF32 %.3e / %.3e, SIMT %.3e / %.3e" % (e_tf, m_tf, e_simt, m_simt))
    assert e_tf <= 1e-6 and e_simt <= 1e-6
    assert m_tf <= 2e-6
    np.testing.assert_allclose(parts, want_parts, rtol=2e-6)
    ctx.close()


def test_tf32_defaults_and_bias_under_strong_scattering(kgb):
    """The mixed default runs the TF32 LPlusTimes and the SIMT LTimes.  On a problem with
    scattering ratios up to 0.9 (one of the seeded uneven batch problems: 27 x 37 x 15 zones, 32
    groups, 48 directions, P4), after 10 iterations, the default's phi error against FP64 stays
    within 1.6x the all-SIMT error (the leading moment added last), while the TF32 LTimes, opt-in,
    shows the bias of its truncating accumulations."""
    from kripke_gb300.batching import uneven_inputs
    im, idd = uneven_inputs(48, seed=2026, precision=kgb.MIXED)[18], uneven_inputs(48, seed=2026, precision=kgb.FP64)[18]
    c = kgb.Context(0)
    c.generate(idd)
    c.solve(10)
    ref = c.download("phi")
    c.close()
    errs = {}
    for name, opts in (("default", {}), ("simt", {"moments_tf32": 0}), ("tf32_lt", {"moments_tf32_ltimes": 1})):
        c = kgb.Context(0)
        c.generate(im)
        for k, v in opts.items():
            c.set_option(k, v)
        c.solve(10)
        errs[name] = (np.linalg.norm(c.download("phi") - ref) / np.linalg.norm(ref),
                      c.get_option("moments_tf32_ltimes"), c.get_option("moments_tf32_lplustimes"))
        c.close()
    print("phi error vs FP64 (2-norm):", {k: "%.3e" % v[0] for k, v in errs.items()})
    assert errs["default"][1:] == (0, 1) and errs["simt"][1:] == (0, 0) and errs["tf32_lt"][1:] == (1, 1)
    assert errs["default"][0] <= 1.6 * errs["simt"][0] and errs["default"][0] <= 1e-6
    assert errs["tf32_lt"][0] <= 1e-6


def test_tf32_not_in_fp64(kgb, oracle):
    p, ctx = pair(oracle, kgb, precision=kgb.FP64, quad=(8, 16), legendre=4)
    assert ctx.get_option("moments_tf32_ltimes") == 0 and ctx.get_option("moments_tf32_lplustimes") == 0
    ctx.close()
