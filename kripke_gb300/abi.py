"""ctypes binding of libkgb.so (include/kgb.h).

The library is built in-tree (kripke_gb300/lib/libkgb.so) by
kripke_gb300.build.  Loading fails loudly when it is missing: there is no
CPU fallback for the GPU path.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libkgb.so")

KGB_OK = 0
STATUS = {0: "KGB_OK", 1: "KGB_ERR_ARG", 2: "KGB_ERR_CUDA", 3: "KGB_ERR_OOM", 4: "KGB_ERR_TIMEOUT",
          5: "KGB_ERR_LAYOUT", 6: "KGB_ERR_STATE"}
LAYOUTS = ("DGZ", "DZG", "GDZ", "GZD", "ZDG", "ZGD")
FP64, MIXED = 0, 1

# Every symbol include/kgb.h declares (checked by tests/test_abi.py).
EXPORTS = (
    "kgb_ctx_create", "kgb_ctx_destroy", "kgb_last_error", "kgb_version", "kgb_setup", "kgb_num_subdomains",
    "kgb_field_bytes", "kgb_field_upload", "kgb_field_download", "kgb_field_fill", "kgb_ltimes",
    "kgb_lplustimes", "kgb_scattering", "kgb_source", "kgb_sweep_subdomain", "kgb_sweep_solver",
    "kgb_population", "kgb_balance", "kgb_solve", "kgb_iterate", "kgb_sync", "kgb_set_stream",
    "kgb_set_option", "kgb_set_timing", "kgb_kernel_time", "kgb_reset_timers", "kgb_default_input",
    "kgb_generate", "kgb_launch_count", "kgb_population_noalloc", "kgb_autotune", "kgb_get_option",
    "kgb_material_tables", "kgb_set_materials", "kgb_set_response", "kgb_solve_converged", "kgb_adjoint_solve",
    "kgb_response", "kgb_gradient", "kgb_gradient_unrolled",
    "kgb_batch_create", "kgb_batch_destroy", "kgb_batch_last_error", "kgb_batch_add", "kgb_batch_size",
    "kgb_batch_context", "kgb_batch_set_option", "kgb_batch_get_option", "kgb_batch_autotune", "kgb_batch_solve",
    "kgb_batch_launch_count", "kgb_batch_profile",
)

INT_FIELDS = ("quadrature/id", "quadrature/jd", "quadrature/kd", "zone_to_mixelem", "zone_to_num_mixelem",
              "mixelem_to_zone", "mixelem_to_material", "moment_to_legendre")


class KgbDims(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("num_groups", ctypes.c_int32), ("num_directions", ctypes.c_int32),
        ("legendre_order", ctypes.c_int32), ("num_groupsets", ctypes.c_int32),
        ("num_dirsets", ctypes.c_int32), ("num_zonesets", ctypes.c_int32 * 3),
        ("layout", ctypes.c_int32), ("precision", ctypes.c_int32),
    ]


class KgbInput(ctypes.Structure):
    """InputVariables plus generator options (kgb_input in include/kgb.h)."""
    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("num_directions", ctypes.c_int32), ("num_groups", ctypes.c_int32),
        ("legendre_order", ctypes.c_int32), ("quad_num_polar", ctypes.c_int32),
        ("quad_num_azimuthal", ctypes.c_int32), ("num_groupsets", ctypes.c_int32),
        ("num_dirsets", ctypes.c_int32), ("num_zonesets", ctypes.c_int32 * 3),
        ("layout", ctypes.c_int32), ("precision", ctypes.c_int32),
        ("num_material_subsamples", ctypes.c_int32), ("geometry", ctypes.c_int32),
        ("scatter", ctypes.c_int32), ("perturb", ctypes.c_int32), ("pad_", ctypes.c_int32),
        ("seed", ctypes.c_uint64), ("sigt", ctypes.c_double * 3), ("sigs", ctypes.c_double * 3),
    ]


def make_input(**kw):
    """kgb_input with the reference defaults, overridden by keywords.

    Shorthands: zones=(x,y,z), zsets=(x,y,z), quad=N (dummy S2) or (polar, azimuthal),
    groups, legendre, gset, dset, layout='DGZ', precision, sigt/sigs triples.
    """
    inp = KgbInput()
    load().kgb_default_input(ctypes.byref(inp))
    for k, v in kw.items():
        if k == "zones":
            inp.nx, inp.ny, inp.nz = v
        elif k == "zsets":
            inp.num_zonesets[0], inp.num_zonesets[1], inp.num_zonesets[2] = v
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
        elif k == "legendre":
            inp.legendre_order = v
        elif k == "gset":
            inp.num_groupsets = v
        elif k == "dset":
            inp.num_dirsets = v
        else:
            setattr(inp, k, v)
    return inp


class KgbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS.get(code, code), msg))
        self.code = code


_lib = None


def load():
    """Load libkgb.so; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libkgb.so not built (%s); run `python -m kripke_gb300.build`" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    P, I, I64, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double
    sig = {
        "kgb_ctx_create": ([I, ctypes.POINTER(P)], I),
        "kgb_ctx_destroy": ([P], I),
        "kgb_last_error": ([P], ctypes.c_char_p),
        "kgb_version": ([], ctypes.c_char_p),
        "kgb_setup": ([P, ctypes.POINTER(KgbDims)], I),
        "kgb_num_subdomains": ([P, ctypes.POINTER(ctypes.c_int32)], I),
        "kgb_field_bytes": ([P, ctypes.c_char_p, ctypes.POINTER(I64)], I),
        "kgb_field_upload": ([P, ctypes.c_char_p, P, I64], I),
        "kgb_field_download": ([P, ctypes.c_char_p, P, I64], I),
        "kgb_field_fill": ([P, ctypes.c_char_p, D], I),
        "kgb_ltimes": ([P], I),
        "kgb_lplustimes": ([P], I),
        "kgb_scattering": ([P], I),
        "kgb_source": ([P, D], I),
        "kgb_sweep_subdomain": ([P, ctypes.c_int32], I),
        "kgb_sweep_solver": ([P], I),
        "kgb_population": ([P, ctypes.POINTER(D)], I),
        "kgb_balance": ([P, ctypes.POINTER(D)], I),
        "kgb_solve": ([P, ctypes.c_int32, D, ctypes.POINTER(D)], I),
        "kgb_iterate": ([P, D, ctypes.POINTER(D)], I),
        "kgb_sync": ([P], I),
        "kgb_set_stream": ([P, P], I),
        "kgb_set_option": ([P, ctypes.c_char_p, I64], I),
        "kgb_get_option": ([P, ctypes.c_char_p, ctypes.POINTER(I64)], I),
        "kgb_set_timing": ([P, I], I),
        "kgb_kernel_time": ([P, ctypes.c_char_p, ctypes.POINTER(D), ctypes.POINTER(I64)], I),
        "kgb_reset_timers": ([P], I),
        "kgb_default_input": ([ctypes.POINTER(KgbInput)], None),
        "kgb_generate": ([P, ctypes.POINTER(KgbInput)], I),
        "kgb_launch_count": ([P, ctypes.POINTER(I64)], I),
        "kgb_autotune": ([P, ctypes.POINTER(D), ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)], I),
        "kgb_population_noalloc": ([P, P, P, I64, ctypes.c_int32, ctypes.c_int32, P, P, ctypes.c_char_p,
                                    ctypes.c_int32], I),
        "kgb_material_tables": ([ctypes.POINTER(KgbInput), P, P], I),
        "kgb_set_materials": ([P, P, P], I),
        "kgb_set_response": ([P, P, I64], I),
        "kgb_solve_converged": ([P, D, D, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(D)], I),
        "kgb_adjoint_solve": ([P, D, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(D)], I),
        "kgb_response": ([P, ctypes.POINTER(D)], I),
        "kgb_gradient": ([P, ctypes.POINTER(D), P, P, ctypes.POINTER(D)], I),
        "kgb_gradient_unrolled": ([P, ctypes.c_int32, D, ctypes.c_int32, ctypes.POINTER(D), P, P,
                                   ctypes.POINTER(D)], I),
        "kgb_batch_create": ([I, ctypes.c_int32, ctypes.POINTER(P)], I),
        "kgb_batch_destroy": ([P], I),
        "kgb_batch_last_error": ([P], ctypes.c_char_p),
        "kgb_batch_add": ([P, ctypes.POINTER(KgbInput), ctypes.POINTER(ctypes.c_int32)], I),
        "kgb_batch_size": ([P, ctypes.POINTER(ctypes.c_int32)], I),
        "kgb_batch_context": ([P, ctypes.c_int32, ctypes.POINTER(P)], I),
        "kgb_batch_set_option": ([P, ctypes.c_char_p, I64], I),
        "kgb_batch_get_option": ([P, ctypes.c_char_p, ctypes.POINTER(I64)], I),
        "kgb_batch_autotune": ([P, ctypes.POINTER(D)], I),
        "kgb_batch_solve": ([P, ctypes.c_int32, D, P], I),
        "kgb_batch_launch_count": ([P, ctypes.POINTER(I64)], I),
        "kgb_batch_profile": ([P, ctypes.POINTER(D)], I),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


class Context:
    """One GPU context holding one Kripke problem (see include/kgb.h)."""

    def __init__(self, device=0):
        self.lib = load()
        h = ctypes.c_void_p()
        rc = self.lib.kgb_ctx_create(device, ctypes.byref(h))
        if rc != KGB_OK:
            raise KgbError(rc, "kgb_ctx_create(%d) failed" % device)
        self.h = h
        self.dims = None

    def _check(self, rc, what):
        if rc != KGB_OK:
            raise KgbError(rc, "%s: %s" % (what, self.lib.kgb_last_error(self.h).decode()))

    def close(self):
        if getattr(self, "h", None):
            self.lib.kgb_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def setup(self, nx, ny, nz, groups, directions, legendre, gset=1, dset=8, zsets=(1, 1, 1), layout="DGZ",
              precision=FP64):
        d = KgbDims()
        d.nx, d.ny, d.nz = nx, ny, nz
        d.num_groups, d.num_directions, d.legendre_order = groups, directions, legendre
        d.num_groupsets, d.num_dirsets = gset, dset
        d.num_zonesets[0], d.num_zonesets[1], d.num_zonesets[2] = zsets
        d.layout = LAYOUTS.index(layout) if isinstance(layout, str) else int(layout)
        d.precision = precision
        self._check(self.lib.kgb_setup(self.h, ctypes.byref(d)), "kgb_setup")
        self.dims = d

    def setup_like(self, inp, precision=FP64):
        """Shape from an oracle input structure (same field names as InputVariables)."""
        self.setup(inp.nx, inp.ny, inp.nz, inp.num_groups, inp.num_directions, inp.legendre_order,
                   inp.num_groupsets, inp.num_dirsets, tuple(inp.num_zonesets_dim), inp.layout, precision)

    def generate(self, inp=None, **kw):
        """Kripke::generateProblem: set up the shape and upload every generated input."""
        inp = inp if inp is not None else make_input(**kw)
        self._check(self.lib.kgb_generate(self.h, ctypes.byref(inp)), "kgb_generate")
        self.inp = inp
        return inp

    @property
    def num_subdomains(self):
        n = ctypes.c_int32()
        self._check(self.lib.kgb_num_subdomains(self.h, ctypes.byref(n)), "kgb_num_subdomains")
        return n.value

    def field_bytes(self, name):
        n = ctypes.c_int64()
        self._check(self.lib.kgb_field_bytes(self.h, name.encode(), ctypes.byref(n)), "kgb_field_bytes(%s)" % name)
        return n.value

    def upload(self, name, arr):
        dt = np.int32 if name in INT_FIELDS else np.float64
        a = np.ascontiguousarray(arr, dtype=dt)
        self._check(self.lib.kgb_field_upload(self.h, name.encode(), a.ctypes.data, a.nbytes), "upload(%s)" % name)

    def download(self, name, out=None):
        dt = np.int32 if name in INT_FIELDS else np.float64
        nb = self.field_bytes(name)
        if out is None:
            out = np.empty(nb // np.dtype(dt).itemsize, dtype=dt)
        self._check(self.lib.kgb_field_download(self.h, name.encode(), out.ctypes.data, out.nbytes),
                    "download(%s)" % name)
        return out

    def fill(self, name, value):
        self._check(self.lib.kgb_field_fill(self.h, name.encode(), float(value)), "fill(%s)" % name)

    def ltimes(self):
        self._check(self.lib.kgb_ltimes(self.h), "kgb_ltimes")

    def lplustimes(self):
        self._check(self.lib.kgb_lplustimes(self.h), "kgb_lplustimes")

    def scattering(self):
        self._check(self.lib.kgb_scattering(self.h), "kgb_scattering")

    def source(self, strength=1.0):
        self._check(self.lib.kgb_source(self.h, float(strength)), "kgb_source")

    def sweep_subdomain(self, sdom):
        self._check(self.lib.kgb_sweep_subdomain(self.h, sdom), "kgb_sweep_subdomain")

    def sweep_solver(self):
        self._check(self.lib.kgb_sweep_solver(self.h), "kgb_sweep_solver")

    def population(self):
        v = ctypes.c_double()
        self._check(self.lib.kgb_population(self.h, ctypes.byref(v)), "kgb_population")
        return v.value

    def balance(self):
        out = (ctypes.c_double * 5)()
        self._check(self.lib.kgb_balance(self.h, out), "kgb_balance")
        return list(out)

    def solve(self, niter, source_strength=1.0):
        part = (ctypes.c_double * niter)()
        self._check(self.lib.kgb_solve(self.h, niter, source_strength, part), "kgb_solve")
        return list(part)

    def iterate(self, source_strength=1.0, want_population=True):
        v = ctypes.c_double()
        self._check(self.lib.kgb_iterate(self.h, source_strength, ctypes.byref(v) if want_population else None),
                    "kgb_iterate")
        return v.value if want_population else None

    def sync(self):
        self._check(self.lib.kgb_sync(self.h), "kgb_sync")

    def set_stream(self, stream_ptr):
        self._check(self.lib.kgb_set_stream(self.h, ctypes.c_void_p(stream_ptr)), "kgb_set_stream")

    def set_option(self, key, value):
        self._check(self.lib.kgb_set_option(self.h, key.encode(), int(value)), "kgb_set_option(%s)" % key)

    def get_option(self, key):
        v = ctypes.c_int64()
        self._check(self.lib.kgb_get_option(self.h, key.encode(), ctypes.byref(v)), "kgb_get_option(%s)" % key)
        return v.value

    def set_timing(self, on=True):
        self._check(self.lib.kgb_set_timing(self.h, 1 if on else 0), "kgb_set_timing")

    def kernel_time(self, family):
        ms, n = ctypes.c_double(), ctypes.c_int64()
        self._check(self.lib.kgb_kernel_time(self.h, family.encode(), ctypes.byref(ms), ctypes.byref(n)),
                    "kgb_kernel_time")
        return ms.value, n.value

    def autotune(self):
        """Pick the fastest sweep tile shape for this problem (overwrites psi and the planes)."""
        ms, xy, tz = ctypes.c_double(), ctypes.c_int32(), ctypes.c_int32()
        self._check(self.lib.kgb_autotune(self.h, ctypes.byref(ms), ctypes.byref(xy), ctypes.byref(tz)),
                    "kgb_autotune")
        return {"sweep_ms": ms.value, "sweep_tile_xy": xy.value, "sweep_tile_z": tz.value,
                "ltimes_tensor": self.get_option("moments_tensor_ltimes"),
                "lplustimes_tensor": self.get_option("moments_tensor_lplustimes"),
                "ltimes_tf32": self.get_option("moments_tf32_ltimes"),
                "lplustimes_tf32": self.get_option("moments_tf32_lplustimes")}

    def launch_count(self):
        n = ctypes.c_int64()
        self._check(self.lib.kgb_launch_count(self.h, ctypes.byref(n)), "kgb_launch_count")
        return n.value

    def reset_timers(self):
        self._check(self.lib.kgb_reset_timers(self.h), "kgb_reset_timers")

    # --- converged solves, the adjoint and gradients -----------------------
    def set_materials(self, sigt=None, sigs=None):
        """Cross sections from per-material tables: sigt [3][G], sigs [3][L+1][G][G] (dest, source)."""
        a = None if sigt is None else np.ascontiguousarray(sigt, dtype=np.float64).ravel()
        b = None if sigs is None else np.ascontiguousarray(sigs, dtype=np.float64).ravel()
        self._check(self.lib.kgb_set_materials(self.h, None if a is None else a.ctypes.data,
                                               None if b is None else b.ctypes.data), "kgb_set_materials")

    def set_response(self, det=None):
        """Detector weights per zone, z = (k*ny + j)*nx + i; None = the whole domain."""
        if det is None:
            self._check(self.lib.kgb_set_response(self.h, None, 0), "kgb_set_response")
            return
        a = np.ascontiguousarray(det, dtype=np.float64).ravel()
        self._check(self.lib.kgb_set_response(self.h, a.ctypes.data, a.size), "kgb_set_response")

    def solve_converged(self, source_strength=1.0, tol=1e-12, max_iter=1000):
        it, ch = ctypes.c_int32(), ctypes.c_double()
        self._check(self.lib.kgb_solve_converged(self.h, float(source_strength), float(tol), int(max_iter),
                                                 ctypes.byref(it), ctypes.byref(ch)), "kgb_solve_converged")
        return it.value, ch.value

    def adjoint_solve(self, tol=1e-12, max_iter=1000):
        it, ch = ctypes.c_int32(), ctypes.c_double()
        self._check(self.lib.kgb_adjoint_solve(self.h, float(tol), int(max_iter), ctypes.byref(it),
                                               ctypes.byref(ch)), "kgb_adjoint_solve")
        return it.value, ch.value

    def response(self):
        v = ctypes.c_double()
        self._check(self.lib.kgb_response(self.h, ctypes.byref(v)), "kgb_response")
        return v.value

    def gradient(self):
        """(R, dR/dsigt [3][G], dR/dsigs in-group P0 [3][G], dR/dq) at the current psi and adjoint."""
        G = self.dims.num_groups if self.dims is not None else self.inp.num_groups
        r, q = ctypes.c_double(), ctypes.c_double()
        dt = np.zeros((3, G))
        ds = np.zeros((3, G))
        self._check(self.lib.kgb_gradient(self.h, ctypes.byref(r), dt.ctypes.data, ds.ctypes.data, ctypes.byref(q)),
                    "kgb_gradient")
        return r.value, dt, ds, q.value

    def gradient_unrolled(self, niter, source_strength=1.0, stride=0):
        """(R, dR/dsigt, dR/dsigs, dR/dq) after exactly niter iterations from psi = 0 (checkpointed reverse mode)."""
        G = self.dims.num_groups if self.dims is not None else self.inp.num_groups
        r, q = ctypes.c_double(), ctypes.c_double()
        dt = np.zeros((3, G))
        ds = np.zeros((3, G))
        self._check(self.lib.kgb_gradient_unrolled(self.h, int(niter), float(source_strength), int(stride),
                                                   ctypes.byref(r), dt.ctypes.data, ds.ctypes.data,
                                                   ctypes.byref(q)), "kgb_gradient_unrolled")
        return r.value, dt, ds, q.value


def material_tables(inp):
    """The generator's (sigt [3][G], sigs [3][L+1][G][G]) for a kgb_input."""
    G, L1 = inp.num_groups, inp.legendre_order + 1
    st = np.zeros((3, G))
    sg = np.zeros((3, L1, G, G))
    rc = load().kgb_material_tables(ctypes.byref(inp), st.ctypes.data, sg.ctypes.data)
    if rc != KGB_OK:
        raise KgbError(rc, "kgb_material_tables")
    return st, sg


class BorrowedContext(Context):
    """A batch problem's own context (owned by the batch; not destroyed here)."""

    def __init__(self, lib, handle, inp, batch):
        self.lib = lib
        self.h = handle
        self.dims = None
        self.inp = inp
        self._batch = batch  # keeps the batch alive

    def close(self):
        self.h = None


class Batch:
    """Independent problems advanced together (kgb_batch_* in include/kgb.h)."""

    def __init__(self, device=0, precision=FP64):
        self.lib = load()
        h = ctypes.c_void_p()
        rc = self.lib.kgb_batch_create(device, precision, ctypes.byref(h))
        if rc != KGB_OK:
            raise KgbError(rc, "kgb_batch_create(%d) failed" % device)
        self.h = h
        self.inputs = []

    def _check(self, rc, what):
        if rc != KGB_OK:
            raise KgbError(rc, "%s: %s" % (what, self.lib.kgb_batch_last_error(self.h).decode()))

    def close(self):
        if getattr(self, "h", None):
            self.lib.kgb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, inp=None, **kw):
        inp = inp if inp is not None else make_input(**kw)
        idx = ctypes.c_int32()
        self._check(self.lib.kgb_batch_add(self.h, ctypes.byref(inp), ctypes.byref(idx)), "kgb_batch_add")
        self.inputs.append(inp)
        return idx.value

    def __len__(self):
        n = ctypes.c_int32()
        self._check(self.lib.kgb_batch_size(self.h, ctypes.byref(n)), "kgb_batch_size")
        return n.value

    def context(self, i):
        c = ctypes.c_void_p()
        self._check(self.lib.kgb_batch_context(self.h, i, ctypes.byref(c)), "kgb_batch_context")
        return BorrowedContext(self.lib, c, self.inputs[i], self)

    def set_option(self, key, value):
        self._check(self.lib.kgb_batch_set_option(self.h, key.encode(), int(value)), "kgb_batch_set_option(%s)" % key)

    def get_option(self, key):
        v = ctypes.c_int64()
        self._check(self.lib.kgb_batch_get_option(self.h, key.encode(), ctypes.byref(v)),
                    "kgb_batch_get_option(%s)" % key)
        return v.value

    def autotune(self):
        ms = ctypes.c_double()
        self._check(self.lib.kgb_batch_autotune(self.h, ctypes.byref(ms)), "kgb_batch_autotune")
        return {"iteration_ms": ms.value, "sweep_tile_xy": self.get_option("sweep_tile_xy"),
                "sweep_tile_z": self.get_option("sweep_tile_z"), "rows_per_item": self.get_option("rows_per_item"),
                "per_problem_sweeps": self.get_option("per_problem_sweeps")}

    def solve(self, niter, source_strength=1.0):
        """Particle counts [niter][problems]."""
        out = np.zeros((niter, len(self)))
        self._check(self.lib.kgb_batch_solve(self.h, int(niter), float(source_strength), out.ctypes.data),
                    "kgb_batch_solve")
        return out

    def launch_count(self):
        n = ctypes.c_int64()
        self._check(self.lib.kgb_batch_launch_count(self.h, ctypes.byref(n)), "kgb_batch_launch_count")
        return n.value

    def profile(self):
        """Device ms per phase of one iteration: ltimes, scattering, lplustimes, sweep, population."""
        ms = (ctypes.c_double * 5)()
        self._check(self.lib.kgb_batch_profile(self.h, ms), "kgb_batch_profile")
        return dict(zip(("ltimes", "scattering", "lplustimes", "sweep", "population"), list(ms)))
