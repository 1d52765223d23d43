"""Build recipe for libkgb.so (the C ABI in include/kgb.h) and the kripke CLI.

Every CUDA translation unit is compiled for sm_103a only, in parallel, and
linked in-tree into kripke_gb300/lib/.  Host C++ is compiled with
-ffp-contract=off so host-side arithmetic (problem generation, coefficient
tables) rounds the same way on x86-64 and aarch64.

    python -m kripke_gb300.build          # build if sources changed
    python -m kripke_gb300.build --force  # rebuild everything
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(CSRC, "host")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
BINDIR = os.path.join(HERE, "bin")
LIB = os.path.join(LIBDIR, "libkgb.so")
CLI = os.path.join(BINDIR, "kripke")
PROBE = os.path.join(BINDIR, "peak_probe")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + os.path.join(ROOT, "include"),
]
CUDA_INCLUDE = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")  # NVTX (header-only)
CXX_FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-Wall", "-I" + os.path.join(ROOT, "include"),
             "-I" + HOST, "-I" + CUDA_INCLUDE]

CU_SOURCES = ["kgb_context.cu", "kgb_solver.cu", "kgb_adjoint_api.cu", "kgb_options.cu", "sweep.cu", "moments.cu", "scatter.cu", "reduce.cu", "xpose.cu", "noalloc.cu", "tc_moments.cu",
              "adjoint.cu", "batch.cu", "tf32_moments.cu", "sweep_stream.cu", "ltimes_stream.cu"]
CPP_SOURCES = ["generate.cpp"]
HEADERS = ["kgb_ctx.h", "kgb_internal.h", "kgb_layout.h", "exact_round.h", "sweep_common.h", "fp32_pair.h", "ltimes_sym.h"]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n  %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _host_sources():
    if not os.path.isdir(HOST):
        return []
    return sorted(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".cpp"))


def build(force=False, verbose=False):
    """Compile libkgb.so (and the kripke CLI if its sources exist); return the library path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "kgb.h")]
    jobs, objs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cpp", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append(["g++"] + CXX_FLAGS + ["-I" + CSRC, "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    if force or jobs or _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    os.makedirs(BINDIR, exist_ok=True)
    probe_src = os.path.join(CSRC, "tools", "peak_probe.cu")
    if force or _stale(PROBE, [probe_src]):
        _run([nvcc] + ARCH + ["-O3", "-std=c++17", "-o", PROBE, probe_src])
    host = _host_sources()
    if host:
        os.makedirs(BINDIR, exist_ok=True)
        hhdrs = [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")]
        if force or _stale(CLI, host + hhdrs + [LIB]):
            _run(["g++"] + CXX_FLAGS + ["-o", CLI] + host +
                 ["-L" + LIBDIR, "-lkgb", "-Wl,-rpath,$ORIGIN/../lib", "-ldl"])
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
