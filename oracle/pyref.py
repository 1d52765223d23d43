"""ctypes binding of the REFERENCE's own code built by oracle/ref_build.sh (oracle/_ref/).

TEST INFRASTRUCTURE ONLY: the reference's generator, Kernel::* functions, SweepSolver and
SteadyStateSolver, compiled from its sources, used to pin the oracle (tests/test_ref_pin.py and
tests/golden/make_ref_fixtures.py).  The product never imports it.  The library exists only where
the reference sources were present at build time; `available()` says whether it can be loaded.
"""
import ctypes
import os
import subprocess

import numpy as np

from oracle import pyoracle

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libkripke_ref.so")
CLI_PATH = os.path.join(_HERE, "_ref", "kripke")
_lib = None


def build(src=None):
    """Compile the reference's sources with oracle/ref_build.sh; False if they are absent."""
    cmd = ["sh", os.path.join(_HERE, "ref_build.sh")] + ([src] if src else [])
    return subprocess.run(cmd, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL).returncode == 0


def available():
    try:
        lib()
        return True
    except OSError:
        return False


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        L.ref_create.argtypes = [ctypes.POINTER(pyoracle.OrcInput)]
        L.ref_create.restype = P
        L.ref_destroy.argtypes = [P]
        L.ref_error.restype = ctypes.c_char_p
        L.ref_set_quiet.argtypes = [P, ctypes.c_int]
        L.ref_set_block_jacobi.argtypes = [P, ctypes.c_int]
        L.ref_field_size.argtypes = [P, ctypes.c_char_p]
        L.ref_field_size.restype = ctypes.c_int64
        L.ref_field_elem_bytes.argtypes = [P, ctypes.c_char_p]
        L.ref_field_elem_bytes.restype = ctypes.c_int32
        L.ref_field_get.argtypes = [P, ctypes.c_char_p, P]
        L.ref_field_set.argtypes = [P, ctypes.c_char_p, P]
        L.ref_kconst.argtypes = [P, ctypes.c_char_p, ctypes.c_double]
        for n in ("ref_ltimes", "ref_lplustimes", "ref_scattering", "ref_source", "ref_sweep_solver", "ref_num_sdoms"):
            getattr(L, n).argtypes = [P]
            getattr(L, n).restype = ctypes.c_int32
        L.ref_sweep_subdomain.argtypes = [P, ctypes.c_int32]
        L.ref_sweep_subdomain.restype = ctypes.c_int32
        L.ref_population.argtypes = [P]
        L.ref_population.restype = ctypes.c_double
        L.ref_solve.argtypes = [P, ctypes.c_int32, ctypes.POINTER(ctypes.c_double)]
        L.ref_solve.restype = ctypes.c_int32
        _lib = L
    return _lib


class Problem:
    """One problem generated and held by the reference's own DataStore (sequential policies)."""

    def __init__(self, inp=None, block_jacobi=False, **kw):
        self.inp = inp if inp is not None else pyoracle.default_input(**kw)
        self.h = lib().ref_create(ctypes.byref(self.inp))
        if not self.h:
            raise ValueError("reference rejected input: " + lib().ref_error().decode())
        if block_jacobi:
            lib().ref_set_block_jacobi(self.h, 1)

    def close(self):
        if self.h:
            lib().ref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_sdoms(self):
        return lib().ref_num_sdoms(self.h)

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(lib().ref_error().decode())

    def get(self, name):
        n = lib().ref_field_size(self.h, name.encode())
        if n < 0:
            raise KeyError(name)
        eb = lib().ref_field_elem_bytes(self.h, name.encode())
        arr = np.empty(n, dtype=np.int32 if eb == 4 else np.float64)
        self._check(lib().ref_field_get(self.h, name.encode(), arr.ctypes.data))
        return arr

    def set(self, name, values):
        n = lib().ref_field_size(self.h, name.encode())
        eb = lib().ref_field_elem_bytes(self.h, name.encode())
        arr = np.ascontiguousarray(values, dtype=np.int32 if eb == 4 else np.float64).ravel()
        if arr.size != n:
            raise ValueError("size mismatch for %s: %d != %d" % (name, arr.size, n))
        self._check(lib().ref_field_set(self.h, name.encode(), arr.ctypes.data))

    def kconst(self, name, value):
        self._check(lib().ref_kconst(self.h, name.encode(), value))

    def ltimes(self):
        self._check(lib().ref_ltimes(self.h))

    def lplustimes(self):
        self._check(lib().ref_lplustimes(self.h))

    def scattering(self):
        self._check(lib().ref_scattering(self.h))

    def source(self):
        self._check(lib().ref_source(self.h))

    def sweep_subdomain(self, sdom):
        self._check(lib().ref_sweep_subdomain(self.h, sdom))

    def sweep_solver(self):
        self._check(lib().ref_sweep_solver(self.h))

    def population(self):
        return lib().ref_population(self.h)

    def solve(self, niter=None):
        """Kripke::SteadyStateSolver from psi = 0; returns the final iterate's population."""
        niter = self.inp.niter if niter is None else niter
        part = ctypes.c_double(0.0)
        self._check(lib().ref_solve(self.h, niter, ctypes.byref(part)))
        return part.value
