"""Seeded sets of uneven problems for the batched driver.

Each problem is the 100 cm three-material cube with seeded lower-triangular
downscatter; per problem the zones per axis, groups, directions (Gauss-Legendre
product sets) and Legendre order are drawn from the given choices, and per
material sigma_t and the scattering ratio sigma_s / sigma_t from the given
ranges.
"""
import numpy as np

from . import abi

# directions -> (polar, azimuthal) of the product quadrature
PRODUCT_SETS = {32: (4, 8), 48: (4, 12), 64: (4, 16), 96: (8, 12), 128: (8, 16), 192: (8, 24)}


def uneven_inputs(n, seed=2026, zones=(8, 48), groups=(8, 16, 32, 64), directions=(48, 96, 192), legendre=(2, 4),
                  sigt=(0.05, 0.5), ratio=(0.3, 0.9), precision=abi.FP64):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        nx, ny, nz = (int(v) for v in rng.integers(zones[0], zones[1] + 1, size=3))
        G = int(rng.choice(groups))
        D = int(rng.choice(directions))
        L = int(rng.choice(legendre))
        st = rng.uniform(sigt[0], sigt[1], size=3)
        c = rng.uniform(ratio[0], ratio[1], size=3)
        inp = abi.make_input(zones=(nx, ny, nz), groups=G, quad=PRODUCT_SETS[D], legendre=L, gset=1, dset=8,
                             geometry=1, scatter=1, sigt=tuple(st), sigs=tuple(st * c), precision=precision,
                             seed=int(rng.integers(1, 2 ** 62)))
        out.append(inp)
    return out


def unknowns(inp):
    return inp.nx * inp.ny * inp.nz * inp.num_groups * inp.num_directions
