"""Elementwise error of the FP64 tensor-core moment transforms and scattering.

The exact-digit tensor-core kernels (tc_moments.cu) scale each row by its own largest exponent and
keep 54 bits of every element relative to it, form the digit products exactly and round once per
output.  Here each output is held to the dot-product bound of its own terms,

    |C_gpu - C_oracle| <= 2 K 2^-52 sum_k |a_k| |b_k|,

not to a fraction of the largest output: at the shape of the 64^3 workload (64 groups, 128
Gauss-Legendre directions, Legendre order 4) on 16^3 zones, with (zone, group) rows scaled by
factors spanning 20 decades, and inputs built so that every higher moment nearly cancels (psi
isotropic to 1e-6 within a row, so sum_d ell(m, d) psi(d) for m > 0 is about 1e-6 of sum |ell||psi|).
The oracle's own sum order contributes at most K 2^-53 sum |a||b| of the allowance.
Reference kernels: Kernel/LTimes.cpp:60-64, Kernel/LPlusTimes.cpp:55-59, Kernel/Scattering.cpp:79-98.
"""
import numpy as np
import pytest

from tests.test_gpu_parity import pair

pytestmark = pytest.mark.gpu

SHAPE = dict(zones=(16, 16, 16), groups=64, quad=(8, 16), legendre=4, gset=1, dset=8, geometry=1, scatter=1)


def check(got, want, absdot, K, what):
    bound = 2.0 * K * 2.0 ** -52 * absdot
    err = np.abs(got - want)
    worst = np.max(err / np.maximum(absdot, 1e-300))
    assert np.all(err <= bound), "%s: worst error %.3e of sum|a||b| (bound %.3e)" % (what, worst, 2 * K * 2.0 ** -52)
    return worst


def test_digit_products_elementwise(oracle, kgb):
    p, ctx = pair(oracle, kgb, **SHAPE)
    assert ctx.get_option("moments_tensor") == 1
    rng = np.random.default_rng(2027)
    Z, G, D, M = 16 ** 3, 64, 128, 25
    # host nesting DGZ, one group set, 8 direction sets: psi is [8 sets][16 directions][G][Z]
    row_scale = 10.0 ** rng.uniform(-10.0, 10.0, (G, Z))
    psi = (1.0 + 1e-6 * rng.uniform(-1.0, 1.0, (8, D // 8, G, Z))) * row_scale
    p.set("psi", psi.ravel()); ctx.upload("psi", psi.ravel())
    p.kconst("phi", 0.0); ctx.fill("phi", 0.0)
    p.ltimes(); ctx.ltimes()
    assert ctx.get_option("moments_tensor_ltimes") == 1
    want, got = p.get("phi"), ctx.download("phi")
    ell = p.get("ell")
    p.set("psi", np.abs(psi).ravel()); p.set("ell", np.abs(ell)); p.kconst("phi", 0.0); p.ltimes()
    absdot = p.get("phi")
    p.set("ell", ell)
    wl = check(got, want, absdot, D, "LTimes")
    # the higher moments do cancel: |phi| far below sum |ell||psi| there
    m = want.reshape(M, G, Z)[1:]
    assert np.median(np.abs(m) / absdot.reshape(M, G, Z)[1:]) < 1e-5

    # LPlusTimes: phi_out rows spanning 20 decades, higher moments 1e-3 of moment 0 with either sign
    phi_out = rng.uniform(-1e-3, 1e-3, (M, G, Z))
    phi_out[0] = 1.0
    phi_out *= 10.0 ** rng.uniform(-10.0, 10.0, (G, Z))
    p.set("phi_out", phi_out.ravel()); ctx.upload("phi_out", phi_out.ravel())
    p.kconst("rhs", 0.0); ctx.fill("rhs", 0.0)
    p.lplustimes(); ctx.lplustimes()
    assert ctx.get_option("moments_tensor_lplustimes") == 1
    want, got = p.get("rhs"), ctx.download("rhs")
    ellp = p.get("ell_plus")
    p.set("phi_out", np.abs(phi_out).ravel()); p.set("ell_plus", np.abs(ellp)); p.kconst("rhs", 0.0); p.lplustimes()
    absdot = p.get("rhs")
    p.set("ell_plus", ellp)
    wp = check(got, want, absdot, M, "LPlusTimes")

    # scattering: zones spanning 20 decades, each moment's group spectrum within one decade,
    # either sign (moments above 0 of a nearly isotropic flux)
    phi = (10.0 ** rng.uniform(-1.0, 0.0, (M, G, Z))) * rng.choice([-1.0, 1.0], (M, G, Z))
    phi[0] = np.abs(phi[0])
    phi *= 10.0 ** rng.uniform(-10.0, 10.0, Z)
    p.set("phi", phi.ravel()); ctx.upload("phi", phi.ravel())
    p.kconst("phi_out", 0.0); ctx.fill("phi_out", 0.0)
    p.scattering(); ctx.scattering()
    assert ctx.get_option("scattering_tensor_active") == 1
    want, got = p.get("phi_out"), ctx.download("phi_out")
    sigs = p.get("data/sigs")
    p.set("phi", np.abs(phi).ravel()); p.set("data/sigs", np.abs(sigs)); p.kconst("phi_out", 0.0); p.scattering()
    absdot = p.get("phi_out")
    ws = check(got, want, absdot, G, "scattering")
    print("worst error / sum|a||b|: LTimes %.2e, LPlusTimes %.2e, scattering %.2e (K 2^-52: %.2e, %.2e, %.2e)"
          % (wl, wp, ws, D * 2.0 ** -52, M * 2.0 ** -52, G * 2.0 ** -52))
    ctx.close()
