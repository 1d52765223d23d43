"""Test helper: view Kripke field chunks in logical index order.

A field chunk with index types (T1..Tn) is stored with the types sorted by
their position in the nesting's order list (src/Kripke/VarTypes.h:73-101);
the first sorted index has the longest stride.  These helpers reshape the
concatenated chunks that the oracle and the C ABI exchange into logical
arrays so tests can compare nestings and index by (direction, group, zone).
"""
import numpy as np

ORDER = {
    "DGZ": ["long", "dim", "mat", "dir", "leg", "mom", "ggrp", "grp", "zone", "zk", "zj", "zi", "mix"],
    "DZG": ["long", "dim", "mat", "dir", "leg", "mom", "zone", "zk", "zj", "zi", "ggrp", "grp", "mix"],
    "GDZ": ["long", "dim", "mat", "ggrp", "grp", "dir", "leg", "mom", "zone", "zk", "zj", "zi", "mix"],
    "GZD": ["long", "dim", "mat", "ggrp", "grp", "zone", "zk", "zj", "zi", "mix", "dir", "leg", "mom"],
    "ZDG": ["long", "dim", "mat", "zone", "zk", "zj", "zi", "mix", "dir", "leg", "mom", "ggrp", "grp"],
    "ZGD": ["long", "dim", "mat", "zone", "zk", "zj", "zi", "mix", "ggrp", "grp", "dir", "leg", "mom"],
}
LAYOUTS = tuple(ORDER)

KINDS = {
    "psi": ("dir", "grp", "zone"), "rhs": ("dir", "grp", "zone"),
    "phi": ("mom", "grp", "zone"), "phi_out": ("mom", "grp", "zone"),
    "i_plane": ("dir", "grp", "zj", "zk"), "j_plane": ("dir", "grp", "zi", "zk"),
    "k_plane": ("dir", "grp", "zi", "zj"),
    "ell": ("mom", "dir"), "ell_plus": ("dir", "mom"), "sigt_zonal": ("grp", "zone"),
    "data/sigs": ("mat", "leg", "ggrp", "ggrp"),
}


def strides(layout, types, dims):
    pos = [ORDER[layout].index(t) for t in types]
    order = sorted(range(len(types)), key=lambda i: pos[i])  # stable: ties keep argument order
    st = [0] * len(types)
    s = 1
    for i in reversed(order):
        st[i] = s
        s *= dims[i]
    return st


def chunk_dims(name, info, L=None, G=None):
    Ds, Gs, nx, ny, nz, M = info["Ds"], info["Gs"], info["nxs"], info["nys"], info["nzs"], info["M"]
    Z = nx * ny * nz
    return {
        "psi": (Ds, Gs, Z), "rhs": (Ds, Gs, Z), "phi": (M, Gs, Z), "phi_out": (M, Gs, Z),
        "i_plane": (Ds, Gs, ny, nz), "j_plane": (Ds, Gs, nx, nz), "k_plane": (Ds, Gs, nx, ny),
        "ell": (M, Ds), "ell_plus": (Ds, M), "sigt_zonal": (Gs, Z),
        "data/sigs": (3, (L or 0) + 1, G, G),
    }[name]


def logical_chunks(arr, name, layout, dims, nchunks):
    """Split a concatenated field into nchunks logical arrays of shape dims."""
    n = int(np.prod(dims))
    out = []
    st = strides(layout, KINDS[name], dims)
    for c in range(nchunks):
        flat = arr[c * n:(c + 1) * n]
        out.append(np.lib.stride_tricks.as_strided(flat, shape=dims, strides=[s * flat.itemsize for s in st]).copy())
    return out
