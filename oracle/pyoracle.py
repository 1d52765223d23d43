"""ctypes binding of the CPU oracle (oracle/kripke_oracle.cpp).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py as the checker.  The product package never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libkripke_oracle.so")
_lib = None

LAYOUTS = ("DGZ", "DZG", "GDZ", "GZD", "ZDG", "ZGD")


class OrcInput(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("num_directions", ctypes.c_int32), ("num_groups", ctypes.c_int32),
        ("legendre_order", ctypes.c_int32), ("quad_num_polar", ctypes.c_int32),
        ("quad_num_azimuthal", ctypes.c_int32), ("layout", ctypes.c_int32),
        ("num_dirsets", ctypes.c_int32), ("num_groupsets", ctypes.c_int32),
        ("num_zonesets_dim", ctypes.c_int32 * 3), ("niter", ctypes.c_int32),
        ("num_material_subsamples", ctypes.c_int32), ("geometry", ctypes.c_int32),
        ("scatter", ctypes.c_int32), ("perturb", ctypes.c_int32), ("pad_", ctypes.c_int32),
        ("seed", ctypes.c_uint64), ("sigt", ctypes.c_double * 3), ("sigs", ctypes.c_double * 3),
        ("source_strength", ctypes.c_double),
    ]


def build():
    """Compile the oracle with its Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        L.orc_default_input.argtypes = [ctypes.POINTER(OrcInput)]
        L.orc_create.argtypes = [ctypes.POINTER(OrcInput)]
        L.orc_create.restype = P
        L.orc_destroy.argtypes = [P]
        L.orc_error.restype = ctypes.c_char_p
        L.orc_set_threads.argtypes = [P, ctypes.c_int]
        L.orc_set_block_jacobi.argtypes = [P, ctypes.c_int]
        L.orc_num_sdoms.argtypes = [P]
        L.orc_num_sdoms.restype = ctypes.c_int32
        L.orc_field_size.argtypes = [P, ctypes.c_char_p]
        L.orc_field_size.restype = ctypes.c_int64
        L.orc_field_elem_bytes.argtypes = [P, ctypes.c_char_p]
        L.orc_field_elem_bytes.restype = ctypes.c_int32
        L.orc_field_get.argtypes = [P, ctypes.c_char_p, P]
        L.orc_field_set.argtypes = [P, ctypes.c_char_p, P]
        L.orc_sdom_info.argtypes = [P, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
        L.orc_kconst.argtypes = [P, ctypes.c_char_p, ctypes.c_double]
        for n in ("orc_ltimes", "orc_lplustimes", "orc_scattering", "orc_source", "orc_sweep_solver"):
            getattr(L, n).argtypes = [P]
        L.orc_sweep_subdomain.argtypes = [P, ctypes.c_int32]
        L.orc_population.argtypes = [P]
        L.orc_population.restype = ctypes.c_double
        L.orc_balance.argtypes = [P, ctypes.POINTER(ctypes.c_double)]
        L.orc_solve.argtypes = [P, ctypes.c_int32, ctypes.POINTER(ctypes.c_double)]
        L.orc_iterate.argtypes = [P]
        L.orc_iterate.restype = ctypes.c_double
        L.orc_last_solve_seconds.argtypes = [P]
        L.orc_last_solve_seconds.restype = ctypes.c_double
        _lib = L
    return _lib


def default_input(**kw):
    """InputVariables defaults (src/Kripke/InputVariables.cpp:17-47) with overrides.

    Accepts zones=(x,y,z), zsets=(x,y,z), quad=N or (polar, azim), layout='DGZ', sigt/sigs tuples.
    """
    inp = OrcInput()
    lib().orc_default_input(ctypes.byref(inp))
    for k, v in kw.items():
        if k == "zones":
            inp.nx, inp.ny, inp.nz = v
        elif k == "zsets":
            inp.num_zonesets_dim[0], inp.num_zonesets_dim[1], inp.num_zonesets_dim[2] = v
        elif k == "quad":
            if isinstance(v, (tuple, list)):
                inp.quad_num_polar, inp.quad_num_azimuthal = v
                inp.num_directions = v[0] * v[1]
            else:
                inp.num_directions, inp.quad_num_polar, inp.quad_num_azimuthal = v, 0, 0
        elif k == "layout":
            inp.layout = LAYOUTS.index(v) if isinstance(v, str) else int(v)
        elif k in ("sigt", "sigs"):
            arr = getattr(inp, k)
            for i in range(3):
                arr[i] = v[i]
        elif k == "groups":
            inp.num_groups = v
        elif k == "dset":
            inp.num_dirsets = v
        elif k == "gset":
            inp.num_groupsets = v
        elif k == "legendre":
            inp.legendre_order = v
        else:
            setattr(inp, k, v)
    return inp


class Problem:
    """One generated problem held by the oracle (Kripke DataStore equivalent)."""

    def __init__(self, inp=None, threads=0, block_jacobi=False, **kw):
        self.inp = inp if inp is not None else default_input(**kw)
        self.h = lib().orc_create(ctypes.byref(self.inp))
        if not self.h:
            raise ValueError("oracle rejected input: " + lib().orc_error().decode())
        if threads:
            lib().orc_set_threads(self.h, threads)
        if block_jacobi:
            self.set_block_jacobi(True)

    def set_block_jacobi(self, on):
        """--pmethod bj (SteadyStateSolver's block_jacobi) for every later sweep solve."""
        lib().orc_set_block_jacobi(self.h, 1 if on else 0)

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_sdoms(self):
        return lib().orc_num_sdoms(self.h)

    def sdom_info(self, sdom):
        out = (ctypes.c_int32 * 8)()
        lib().orc_sdom_info(self.h, sdom, out)
        return dict(zip(("Ds", "Gs", "nxs", "nys", "nzs", "glower", "dlower", "M"), list(out)))

    def field_names(self):
        return FIELD_NAMES

    def get(self, name):
        n = lib().orc_field_size(self.h, name.encode())
        if n < 0:
            raise KeyError(name)
        eb = lib().orc_field_elem_bytes(self.h, name.encode())
        arr = np.empty(n, dtype=np.int32 if eb == 4 else np.float64)
        lib().orc_field_get(self.h, name.encode(), arr.ctypes.data)
        return arr

    def set(self, name, values):
        n = lib().orc_field_size(self.h, name.encode())
        eb = lib().orc_field_elem_bytes(self.h, name.encode())
        arr = np.ascontiguousarray(values, dtype=np.int32 if eb == 4 else np.float64).ravel()
        if arr.size != n:
            raise ValueError("size mismatch for %s: %d != %d" % (name, arr.size, n))
        lib().orc_field_set(self.h, name.encode(), arr.ctypes.data)

    def kconst(self, name, value):
        lib().orc_kconst(self.h, name.encode(), value)

    def ltimes(self):
        lib().orc_ltimes(self.h)

    def lplustimes(self):
        lib().orc_lplustimes(self.h)

    def scattering(self):
        lib().orc_scattering(self.h)

    def source(self):
        lib().orc_source(self.h)

    def sweep_subdomain(self, sdom):
        lib().orc_sweep_subdomain(self.h, sdom)

    def sweep_solver(self):
        lib().orc_sweep_solver(self.h)

    def population(self):
        return lib().orc_population(self.h)

    def balance(self):
        out = (ctypes.c_double * 5)()
        lib().orc_balance(self.h, out)
        return list(out)

    def solve(self, niter=None):
        niter = self.inp.niter if niter is None else niter
        part = (ctypes.c_double * niter)()
        lib().orc_solve(self.h, niter, part)
        return list(part)

    def iterate(self):
        return lib().orc_iterate(self.h)

    def last_solve_seconds(self):
        return lib().orc_last_solve_seconds(self.h)


FIELD_NAMES = (
    "psi", "rhs", "phi", "phi_out", "i_plane", "j_plane", "k_plane", "ell", "ell_plus",
    "sigt_zonal", "data/sigs", "quadrature/xcos", "quadrature/ycos", "quadrature/zcos",
    "quadrature/w", "quadrature/id", "quadrature/jd", "quadrature/kd", "dx", "dy", "dz",
    "volume", "zone_to_mixelem", "zone_to_num_mixelem", "mixelem_to_zone",
    "mixelem_to_material", "mixelem_to_fraction", "moment_to_legendre",
)

# inputs the hot path reads (everything generateProblem writes except state)
INPUT_NAMES = tuple(n for n in FIELD_NAMES if n not in ("psi", "rhs", "phi", "phi_out", "i_plane", "j_plane", "k_plane"))
