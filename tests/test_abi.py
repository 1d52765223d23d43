"""The C-ABI library builds, loads and exports every symbol include/kgb.h declares.

Runs without a GPU: no compute call is made, only argument validation and
context creation, which must fail cleanly (KGB_ERR_CUDA) when no device exists.
"""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "kgb.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(kgb_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from kripke_gb300 import build
    build.build()
    from kripke_gb300 import abi
    return abi.load()


def test_header_symbols_exported(lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    from kripke_gb300 import abi
    assert sorted(abi.EXPORTS) == syms
    out = subprocess.run(["nm", "-D", "--defined-only", os.path.join(ROOT, "kripke_gb300", "lib", "libkgb.so")],
                         stdout=subprocess.PIPE, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (kgb_\w+)", out))
    missing = [s for s in syms if s not in exported]
    assert not missing, missing


def test_build_targets_sm103a_only():
    from kripke_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_version_and_null_args(lib):
    assert lib.kgb_version().startswith(b"kripke_gb300")
    assert lib.kgb_ctx_create(0, None) == 1          # KGB_ERR_ARG
    assert lib.kgb_ctx_destroy(None) == 1
    assert lib.kgb_setup(None, None) == 1
    assert lib.kgb_ltimes(None) == 1
    assert lib.kgb_last_error(None) == b"null context"


def test_context_without_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present; covered by the gpu tests")
    h = ctypes.c_void_p()
    assert lib.kgb_ctx_create(0, ctypes.byref(h)) == 2   # KGB_ERR_CUDA
    assert not h.value


def test_python_binding_fails_loudly_without_library(monkeypatch, tmp_path):
    from kripke_gb300 import abi
    monkeypatch.setattr(abi, "_lib", None)
    monkeypatch.setattr(abi, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(ImportError):
        abi.load()
