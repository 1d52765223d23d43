#!/usr/bin/env python
"""Throughput of Kripke's source iteration on GB300 (and the CPU reference arm).

Metric (src/kripke.cpp:495-503): unknowns / (seconds per source iteration),
unknowns = zones * groups * directions.  A "step" is one source iteration
(LTimes, scattering, source, LPlusTimes, full sweep of all octants,
population) over the whole problem, with every field resident in HBM.

Workload at N=1: the plain FP64 GPU drop-in problem -- 64^3 zones on the
100 cm three-material cube, 64 groups, 128 Gauss-Legendre directions (16 per
octant), Legendre order 4, seeded lower-triangular downscatter, DGZ host
nesting, 1 group set, 8 direction sets.  psi and rhs are 17.2 GB each, far
larger than L2, so no L2 flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--precision fp64|mixed]

The FP64 line also carries, from the same run, the mixed form on the same
workload ("mixed": throughput, speed-up over FP64, phi error against FP64
after 20 iterations), the adjoint report ("adjoint": gradient/forward time
and central-difference check at 32^3 zones x 32 groups x 96 directions) and
the batching form ("batch": 48 uneven problems in one graph-replayed solve,
mixed and FP64, against solving them one by one).

--gpus N > 1 (under torchrun) runs N independent replicas, one per GPU
(the path has no data exchange); value = all replicas' unknowns / max time.
--impl reference times the CPU restatement of the reference's OpenMP path
(oracle/) on the host cores, on a bounded sample of the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(zones=(64, 64, 64), groups=64, quad=(8, 16), legendre=4, gset=1, dset=8, geometry=1, scatter=1,
                layout="DGZ")
WORKLOAD_NAME = "kripke 64^3 zones x 64 groups x 128 GL directions, P4, cube100, downscatter, DGZ, dset 8"
# bounded CPU sample: same physics and per-zone work, 32^3 zones (1/8 of the unknowns)
CPU_SAMPLE = dict(WORKLOAD, zones=(32, 32, 32))
# source iterations from psi = 0 before the autotuner times the kernels: the first
# iterates are mostly zero away from the source, which favours other tiles than
# the steady state the timed iterations run in
AUTOTUNE_ITERS = 4
FP64_PEAK_GFLOPS = 1196.0  # DFMA rate kripke_gb300/bin/peak_probe measured on a GB300 at 2,070 MHz (fallback only)
MIXED_PHI_ITERS = 20  # the mixed form's phi error is taken against FP64 after this many iterations
# adjoint gradient workload: cross sections of the reference problem, +-20% per group, isotropic P0
ADJ_WORKLOAD = dict(zones=(32, 32, 32), groups=32, quad=96, legendre=4, gset=1, dset=8, geometry=1, scatter=0,
                    perturb=1, layout="DGZ")
BATCH_PROBLEMS = 48
BATCH_NAME = ("48 independent problems (seed 2026): zones per axis uniform in [8,48], groups from {8,16,32,64}, "
              "directions from {48,96,192} (Gauss-Legendre product sets), Legendre order from {2,4}; cube100 "
              "geometry, per-material sigma_t in [0.05,0.5]/cm, scattering ratio in [0.3,0.9], seeded downscatter")
ADJ_NAME = ("32^3 zones x 32 groups x 96 directions, P4, cube100, isotropic P0 with +-20% per-group perturbation; "
            "absorption in the detector block [80,100]^3 cm")


def fp64_peak(device=0):
    """FP64 FMA rate of this GPU from kripke_gb300/bin/peak_probe, with the SM clock sampled while it
    ran (so the roof can be audited as rate / clock); the recorded figure if the probe cannot run."""
    probe = os.path.join(ROOT, "kripke_gb300", "bin", "peak_probe")
    clocks = ClockSampler(device)
    try:
        clocks.start()
        out = subprocess.run([probe], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, timeout=60)
        clk = clocks.stop()
        v = json.loads(out.stdout.strip().splitlines()[-1])["fp64_fma_gflops"]
        return float(v), "measured live by kripke_gb300/bin/peak_probe (MEASURED_PEAKS.json has no FP64 figure)", clk
    except Exception:
        clocks.stop()
        return FP64_PEAK_GFLOPS, "recorded peak_probe figure at 2,070 MHz (the probe could not run)", None


def unknowns(w):
    z = w["zones"][0] * w["zones"][1] * w["zones"][2]
    q = w["quad"]
    d = q[0] * q[1] if isinstance(q, tuple) else q
    return z * w["groups"] * d


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "_fallback": True}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic(w, prec_bytes):
    """Per-iteration algorithmic flops and bytes per kernel family (inputs read once, outputs written once)."""
    Z = w["zones"][0] * w["zones"][1] * w["zones"][2]
    G = w["groups"]
    q = w["quad"]
    D = q[0] * q[1] if isinstance(q, tuple) else q
    M = (w["legendre"] + 1) ** 2
    U = Z * G * D
    t = prec_bytes
    lower = G * (G + 1) // 2 if w.get("scatter") == 1 else G
    return {
        "ltimes": {"flops": 2.0 * M * D * G * Z, "bytes": (D + M) * G * Z * t},
        "lplustimes": {"flops": 2.0 * M * D * G * Z, "bytes": (D + M) * G * Z * t},
        "scattering": {"flops": 2.0 * M * Z * lower, "bytes": 2.0 * M * G * Z * t},
        # 13 flops + one divide (counted as 4) per unknown; rhs read, psi written, sigma_t per octant
        "sweep": {"flops": 17.0 * U, "bytes": 2.0 * U * t + 8.0 * G * Z * t},
        "population": {"flops": 2.0 * U, "bytes": 1.0 * U * t},
        "source": {"flops": 0.0, "bytes": 0.0},
    }


def cpu_run(sample, threads, warmup, steps):
    from oracle import pyoracle
    p = pyoracle.Problem(threads=threads, **sample)
    p.kconst("psi", 0.0)
    for _ in range(warmup):
        p.iterate()
    t0 = time.perf_counter()
    for _ in range(steps):
        p.iterate()
    dt = (time.perf_counter() - t0) / steps
    return unknowns(sample) / dt, dt


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("KGB_BENCH_BACKEND") != "gloo" else "gloo")
    return world, rank, local


def max_over_ranks(value, world):
    """The largest value over all ranks (the timed region ends when the slowest replica does)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, world, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    sample = dict(CPU_SAMPLE, zones=(args.zones,) * 3) if args.zones else CPU_SAMPLE
    sample_name = ("%d^3-zone sample of the workload (same groups, directions, order, physics), 1 iteration per step"
                   % sample["zones"][0])
    value, dt = cpu_run(sample, threads, args.warmup, args.steps)
    line = {
        "impl": "reference", "metric": "unknowns/s per source iteration", "value": value,
        "unit": "unknowns/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded generator, no external data)",
        "config": {"workload": WORKLOAD_NAME, "sample": sample_name},
        "cpu_baseline": {"value": value, "unit": "unknowns/s", "cores": threads, "kind": "port",
                         "sample": sample_name},
        "e2e": {"value": value, "unit": "unknowns/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def progress(msg):
    """One line on stderr per section, so a slow section can be told from a stuck one."""
    print("[bench %.1fs] %s" % (time.perf_counter() - T0, msg), file=sys.stderr, flush=True)


T0 = time.perf_counter()


def timed_steps(ctx, stream, steps):
    """K source iterations between CUDA events on the stream the kernels run on; ms per iteration."""
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        ctx.iterate(want_population=False)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def timed_solve(ctx, stream, steps):
    """One solve of K iterations (the replayed solve graph) between CUDA events; ms per iteration."""
    import torch
    ctx.solve(steps)  # captures the graph
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    ctx.solve(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def mixed_report(args, local, w, fp64_ctx, fp64_ms):
    """The mixed form on the same workload: throughput against the FP64 form and phi error against FP64."""
    import numpy as np
    import torch
    from kripke_gb300 import abi
    ctx = abi.Context(local)
    ctx.generate(precision=abi.MIXED, **w)
    stream = torch.cuda.Stream(device=local)
    ctx.set_stream(stream.cuda_stream)
    ctx.fill("psi", 0.0)
    for _ in range(AUTOTUNE_ITERS):
        ctx.iterate(want_population=False)
    tuned = ctx.autotune() if not args.no_autotune else None
    ctx.fill("psi", 0.0)
    for _ in range(args.warmup):
        ctx.iterate(want_population=False)
    ms = timed_steps(ctx, stream, args.steps)
    # per-family times (CUDA events around each family on the context's stream) over the same
    # number of further iterations, and each family's algorithmic bytes against the copy bandwidth
    ctx.reset_timers()
    ctx.set_timing(True)
    timed_steps(ctx, stream, args.steps)
    fam_ms = {f: ctx.kernel_time(f)[0] / args.steps for f in ("sweep", "ltimes", "lplustimes", "scattering",
                                                              "source", "population")}
    ctx.set_timing(False)
    alg = algorithmic(w, 4)
    hbm = peaks()["hbm_gbs"]
    traffic = {}
    traffic_file = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(traffic_file):
        traffic = json.load(open(traffic_file))
    fam_roof = {}
    for f in ("sweep", "ltimes", "lplustimes", "scattering"):
        if fam_ms[f] > 0:
            gbs = alg[f]["bytes"] / (fam_ms[f] * 1e-3) / 1e9
            fam_roof[f] = {"achieved_gbs": gbs, "frac_of_hbm": gbs / hbm, "algorithmic_bytes": alg[f]["bytes"],
                           "traffic": traffic.get("mixed/" + f)}
    # the fused LTimes epilogue acts inside a solve (the next iteration takes the sweep's moments):
    # solves of K iterations with and without it
    ms_solve = timed_solve(ctx, stream, args.steps)
    ctx.set_option("fused_ltimes", 1)
    lt_active = ctx.get_option("fused_ltimes_active")
    ms_lt = timed_solve(ctx, stream, args.steps)
    ctx.solve(MIXED_PHI_ITERS)
    phi_lt = ctx.download("phi")
    ctx.set_option("fused_ltimes", 0)
    # the fused sweep (rhs formed inside the sweep, no LPlusTimes launch) on the same state
    ctx.set_option("fused_sweep", 1)
    for _ in range(args.warmup):
        ctx.iterate(want_population=False)
    ms_fused = timed_steps(ctx, stream, args.steps)
    fused_active = ctx.get_option("fused_sweep_active")
    parts_fused = ctx.solve(MIXED_PHI_ITERS)
    phi_fused = ctx.download("phi")
    ctx.set_option("fused_sweep", 0)
    kernels = {k: ctx.get_option(k) for k in ("sweep_tile_xy", "sweep_tile_z", "moments_tf32_ltimes",
                                              "moments_tf32_lplustimes", "moments_tensor_ltimes",
                                              "moments_tensor_lplustimes", "scattering_tensor_active",
                                              "scattering_block_active", "ltimes_symmetric_active")}
    parts = ctx.solve(MIXED_PHI_ITERS)
    fp64_ctx.solve(MIXED_PHI_ITERS)
    a, b = fp64_ctx.download("phi"), ctx.download("phi")
    # the fused sweep forms rhs with the SIMT LPlusTimes arithmetic: compare with that unfused iteration
    ctx.set_option("moments_tf32", 0)
    parts_simt = ctx.solve(MIXED_PHI_ITERS)
    fused_same = bool(np.array_equal(parts_simt, parts_fused) and np.array_equal(ctx.download("phi"), phi_fused))
    del phi_fused
    err = float(np.abs(b - a).max() / np.abs(a).max())
    err_l2 = float(np.linalg.norm(b - a) / np.linalg.norm(a))
    lt_err = phi_errors(phi_lt, a)
    del phi_lt
    # moment 0 (DGZ host nesting: phi chunks are [M][G][Z], one chunk per group set)
    M = (w["legendre"] + 1) ** 2
    a0, b0 = a.reshape(M, -1)[0], b.reshape(M, -1)[0]
    err0 = float(np.abs(b0 - a0).max() / np.abs(a0).max())
    del a, b, a0, b0
    out = {"value": unknowns(w) / (ms * 1e-3), "unit": "unknowns/s", "ms_per_step": ms,
           "speedup_vs_fp64": fp64_ms / ms, "phi_rel_err_vs_fp64": err, "phi_rel_err_l2": err_l2,
           "kernel_ms_per_step": fam_ms,
           "roofline": {"peak_gbs": hbm, "bytes": "algorithmic: inputs read once, outputs written once (the "
                                                   "sweep's entering and leaving faces not counted)",
                        "families": fam_roof},
           "phi0_rel_err_max": err0,
           "phi_err_definition": "after %d iterations from psi = 0: max|phi_mixed - phi_fp64| / max|phi_fp64| over "
                                 "all moments, groups and zones; also the 2-norm ratio and the max-abs relative "
                                 "error of moment 0" % MIXED_PHI_ITERS,
           "autotuned": tuned,
           "kernels": kernels,
           "fused_sweep": {"ms_per_step": ms_fused, "value": unknowns(w) / (ms_fused * 1e-3),
                           "speedup_vs_unfused": ms / ms_fused, "active": fused_active,
                           "identical_to_unfused_simt": fused_same,
                           "what": "LPlusTimes formed inside the sweep (rhs neither written nor read), same tiles; "
                                   "compared bit for bit with the unfused iteration whose LPlusTimes is the SIMT "
                                   "kernel (same arithmetic)"},
           "fused_ltimes": {"ms_per_iteration": ms_lt, "unfused_ms_per_iteration": ms_solve,
                            "speedup_vs_unfused": ms_solve / ms_lt, "active": lt_active,
                            "phi_rel_err_vs_fp64": lt_err,
                            "what": "solves of %d iterations (replayed graphs): every sweep but the last adds the "
                                    "next iteration's moments phi = L psi (FP32 reductions per k-slice of a tile) "
                                    "and the next iteration runs no LTimes" % args.steps}}
    ctx.close()
    return out


def phi_errors(got, want):
    """max|got - want| / max|want| and the 2-norm ratio."""
    import numpy as np
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    d = got - want
    return {"max_rel": float(np.abs(d).max() / np.abs(want).max()),
            "l2_rel": float(np.linalg.norm(d) / np.linalg.norm(want))}


# the CPU configuration (16^3 zones on the cube, 32 identical groups, 96 directions, P4, 10 iterations)
C0 = dict(zones=(16, 16, 16), groups=32, legendre=4, gset=1, dset=8, geometry=1, scatter=0, layout="DGZ")
C0_ITERS = 10
PARITY_TOL = {"fp64": 1e-12, "mixed": 1e-6}


def fp64_parity(local, w, niter, threads, with_mixed):
    """One problem solved by the FP64 GPU path and by the oracle (which reproduces the reference's own
    code bit for bit; tests/test_ref_pin.py): phi, every iteration's particle count and the balance
    terms; optionally the mixed form's phi against both."""
    import numpy as np
    from kripke_gb300 import abi
    from oracle import pyoracle
    ctx = abi.Context(local)
    ctx.generate(**w)
    part = ctx.solve(niter)
    phi = ctx.download("phi")
    bal = ctx.balance()
    ref = pyoracle.Problem(threads=threads, **w)
    rpart = ref.solve(niter)
    rphi = ref.get("phi")
    rbal = ref.balance()
    names = ("emission", "collision", "leakage", "population", "residual")
    out = {"iterations": niter, "phi": phi_errors(phi, rphi),
           "population_max_rel": max(abs(a - b) / abs(b) for a, b in zip(part, rpart)),
           # each balance term's difference relative to the emission (the balance's scale), and to itself
           "balance_rel_vs_emission": {n: abs(bal[i] - rbal[i]) / abs(rbal[0]) for i, n in enumerate(names)},
           "balance_rel_vs_itself": {n: abs(bal[i] - rbal[i]) / abs(rbal[i]) for i, n in enumerate(names)
                                     if n != "residual" and rbal[i] != 0.0},
           "balance_terms": dict(zip(names, rbal))}
    out["balance_max_rel"] = max(out["balance_rel_vs_emission"].values())
    ctx.close()
    if with_mixed:
        m = abi.Context(local)
        m.generate(precision=abi.MIXED, **w)
        m.solve(niter)
        mphi = m.download("phi")
        out["mixed_phi_vs_fp64_gpu"] = phi_errors(mphi, phi)
        out["mixed_phi_vs_oracle"] = phi_errors(mphi, rphi)
        m.close()
    ref.close()
    return out


def parity_report(local, line):
    """Parity of every configuration, in the same run: the FP64 form against the oracle at 1e-12 and
    the mixed form's phi against FP64 at 1e-6."""
    threads = os.cpu_count() or 1
    out = {"tolerance": PARITY_TOL,
           "oracle": "C++ restatement of the reference (oracle/), equal bit for bit to the reference's own "
                     "code on the recorded configurations (tests/test_ref_pin.py, tests/golden/)",
           "errors": "phi: max|d|/max|ref| and 2-norm ratio; populations of every iteration; balance terms"}
    progress("parity: c0, dummy S2")
    out["c0_s2_96"] = fp64_parity(local, dict(C0, quad=96), C0_ITERS, threads, True)
    progress("parity: c0, Gauss-Legendre")
    out["c0_gl_8x12"] = fp64_parity(local, dict(C0, quad=(8, 12)), C0_ITERS, threads, True)
    progress("parity: c1 physics at 32^3")
    out["c1_physics_32cube"] = fp64_parity(local, CPU_SAMPLE, 3, threads, False)
    l2 = {"c0_s2_96": out["c0_s2_96"]["mixed_phi_vs_fp64_gpu"]["l2_rel"],
          "c0_gl_8x12": out["c0_gl_8x12"]["mixed_phi_vs_fp64_gpu"]["l2_rel"]}
    mx = {"c0_s2_96": out["c0_s2_96"]["mixed_phi_vs_fp64_gpu"]["max_rel"],
          "c0_gl_8x12": out["c0_gl_8x12"]["mixed_phi_vs_fp64_gpu"]["max_rel"]}
    if "mixed" in line:
        l2["c2"], mx["c2"] = line["mixed"]["phi_rel_err_l2"], line["mixed"]["phi_rel_err_vs_fp64"]
    if "adjoint" in line:
        e = line["adjoint"]["mixed"]["phi_rel_err_vs_fp64"]
        l2["c3_forward"], mx["c3_forward"] = e["l2_rel"], e["max_rel"]
    if "batch" in line:
        e = line["batch"]["mixed_phi_vs_fp64"]
        l2["c4_worst_problem"], mx["c4_worst_problem"] = e["l2_rel_err_max"], e["max_rel_err_max"]
    out["mixed_phi_l2_rel_vs_fp64"] = l2
    out["mixed_phi_max_rel_vs_fp64"] = mx
    out["criterion"] = ("FP64: phi max|d|/max|ref|, every iteration's population and every balance term relative "
                        "to the emission, each <= 1e-12 against the oracle; mixed: phi 2-norm ratio <= 1e-6 "
                        "against FP64 (max-abs relative reported beside it)")
    fp64 = [max(v["phi"]["max_rel"], v["population_max_rel"], v["balance_max_rel"])
            for k, v in out.items() if isinstance(v, dict) and "phi" in v]
    out["fp64_worst"] = max(fp64)
    out["mixed_worst"] = max(l2.values())
    out["mixed_worst_max_abs"] = max(mx.values())
    out["all_within_tolerance"] = bool(out["fp64_worst"] <= PARITY_TOL["fp64"] and
                                       out["mixed_worst"] <= PARITY_TOL["mixed"])
    return out


def adjoint_report(local, fd_params=3):
    """Gradient / forward time and accuracy of the adjoint at the adjoint workload, FP64 and mixed."""
    import numpy as np
    from kripke_gb300 import abi
    from kripke_gb300.response import context_box_detector

    def timed(fn):
        t0 = time.perf_counter()
        r = fn()
        return r, time.perf_counter() - t0

    res = {"workload": ADJ_NAME, "unknowns": unknowns(ADJ_WORKLOAD)}
    grads, phis = {}, {}
    # FP64 solves to 1e-12; the mixed form, whose FP32 change stalls near 1e-7 while the far
    # (detector) region is still converging, runs the FP64 solves' iteration counts
    counts = {}
    for name, prec in (("fp64", abi.FP64), ("mixed", abi.MIXED)):
        ctx = abi.Context(local)
        inp = ctx.generate(precision=prec, **ADJ_WORKLOAD)
        ctx.set_response(context_box_detector(ctx, (80.0, 80.0, 80.0), (100.0, 100.0, 100.0)))
        tol, nf, na = (1e-12, 2000, 2000) if name == "fp64" else (-1.0, counts["fwd"], counts["adj"])
        ctx.solve_converged(1.0, tol, nf)  # builds the tables; untimed
        ctx.adjoint_solve(tol, na)
        (fit, fch), t_fwd = timed(lambda: ctx.solve_converged(1.0, tol, nf))
        phis[name] = ctx.download("phi")
        (ait, ach), t_adj = timed(lambda: ctx.adjoint_solve(tol, na))
        counts = {"fwd": fit, "adj": ait}
        g, t_grad = timed(ctx.gradient)
        grads[name] = g
        r = {"tol": tol if tol >= 0 else "fixed iteration counts", "forward_s": t_fwd, "forward_iters": fit,
             "forward_change": fch if tol >= 0 else None, "adjoint_s": t_adj, "adjoint_iters": ait,
             "adjoint_change": ach if tol >= 0 else None,
             "gradient_assembly_s": t_grad, "grad_over_fwd": (t_adj + t_grad) / t_fwd, "response": g[0]}
        if name == "fp64":
            # central differences (relative step 1e-4) of the GPU forward at the largest gradient entries
            st, sg = abi.material_tables(inp)
            R, dt, ds, dq = g

            def resp(st_, sg_, q=1.0):
                ctx.set_materials(st_, sg_)
                ctx.solve_converged(q, tol, 2000)
                return ctx.response()

            errs = []
            for arr, kind in ((dt, "sigt"), (ds, "sigs")):
                for flat in np.argsort(-np.abs(arr).ravel())[:fd_params]:
                    m, gg = divmod(int(flat), arr.shape[1])
                    s1, s2, g1, g2 = st.copy(), st.copy(), sg.copy(), sg.copy()
                    if kind == "sigt":
                        h = 1e-4 * st[m, gg]
                        s1[m, gg] += h
                        s2[m, gg] -= h
                    else:
                        h = 1e-4 * sg[m, 0, gg, gg]
                        g1[m, 0, gg, gg] += h
                        g2[m, 0, gg, gg] -= h
                    fd = (resp(s1, g1) - resp(s2, g2)) / (2 * h)
                    errs.append({"param": "%s[%d][%d]" % (kind, m, gg), "adjoint": float(arr[m, gg]), "fd": fd,
                                 "rel_err": abs(arr[m, gg] - fd) / abs(fd)})
            fdq = (resp(st, sg, 1.0 + 1e-4) - resp(st, sg, 1.0 - 1e-4)) / 2e-4
            errs.append({"param": "q", "adjoint": dq, "fd": fdq, "rel_err": abs(dq - fdq) / abs(fdq)})
            r["fd_check"] = errs
            r["fd_max_rel_err"] = max(e["rel_err"] for e in errs)
        res[name] = r
        ctx.close()
    res["mixed"]["phi_rel_err_vs_fp64"] = phi_errors(phis["mixed"], phis["fp64"])
    del phis
    ref, got = grads["fp64"], grads["mixed"]
    res["mixed"]["grad_rel_err_vs_fp64"] = max(
        float(np.abs(got[1] - ref[1]).max() / np.abs(ref[1]).max()),
        float(np.abs(got[2] - ref[2]).max() / np.abs(ref[2]).max()), abs(got[3] - ref[3]) / abs(ref[3]))
    return res


def batch_report(local, problems=BATCH_PROBLEMS, niter=10):
    """The batching form: all problems in one graph-replayed solve against each problem run on its own."""
    from kripke_gb300 import abi
    from kripke_gb300.batching import uneven_inputs, unknowns as problem_unknowns
    name = BATCH_NAME if problems == BATCH_PROBLEMS else BATCH_NAME.replace("48 independent", "%d independent" % problems)
    out = {"workload": name, "iterations_per_solve": niter}
    kept = {}
    for name, prec in (("mixed", abi.MIXED), ("fp64", abi.FP64)):
        inputs = uneven_inputs(problems, seed=2026, precision=prec)
        U = sum(problem_unknowns(x) for x in inputs)
        b = abi.Batch(device=local, precision=prec)
        for x in inputs:
            b.add(x)
        progress("batch %s: autotune" % name)
        tune = b.autotune()
        progress("batch %s: solves" % name)
        b.solve(niter)  # captures the solve graph
        l0 = b.launch_count()
        t0 = time.perf_counter()
        b.solve(niter)
        t_batch = (time.perf_counter() - t0) / niter
        kernels = (b.launch_count() - l0) // niter
        phases = b.profile()
        progress("batch %s: one by one" % name)
        t0 = time.perf_counter()
        for i in range(len(b)):
            b.context(i).solve(niter)
        t_seq = (time.perf_counter() - t0) / niter
        out[name] = {"value": U / t_batch, "unit": "unknowns/s", "unknowns": U, "ms_per_iteration": t_batch * 1e3,
                     "graph_active": b.get_option("graph_active"), "kernels_per_iteration": kernels,
                     "per_problem_kernels": b.get_option("per_problem_kernels"),
                     "per_problem_sweeps": b.get_option("per_problem_sweeps"),
                     "branches": b.get_option("branches"),
                     "autotuned": tune, "phase_ms": phases,
                     "one_by_one": {"value": U / t_seq, "ms_per_iteration": t_seq * 1e3,
                                    "how": "each problem's own context, default options, solved in turn"},
                     "speedup_vs_one_by_one": t_seq / t_batch}
        kept[name] = b
    # each problem's mixed phi after the solve against its FP64 context's (same inputs, same iterations)
    errs = [phi_errors(kept["mixed"].context(i).download("phi"), kept["fp64"].context(i).download("phi"))
            for i in range(len(kept["fp64"]))]
    out["mixed_phi_vs_fp64"] = {"problems": len(errs), "iterations": niter,
                                "max_rel_err_max": max(e["max_rel"] for e in errs),
                                "l2_rel_err_max": max(e["l2_rel"] for e in errs)}
    for b in kept.values():
        b.close()
    return out


def run_gpu(args, world, rank, local):
    import ctypes
    import numpy as np
    import torch
    from kripke_gb300 import abi

    torch.cuda.set_device(local)
    precision = abi.MIXED if args.precision == "mixed" else abi.FP64
    w = dict(WORKLOAD)
    if args.zones:
        w["zones"] = (args.zones, args.zones, args.zones)
    ctx = abi.Context(local)
    inp = ctx.generate(precision=precision, **w)
    for kv in args.option:
        k, v = kv.split("=")
        ctx.set_option(k, int(v))
    stream = torch.cuda.Stream(device=local)
    ctx.set_stream(stream.cuda_stream)
    U = unknowns(w)

    # a few source iterations to form a realistic rhs, then the sweep autotuner (untimed set-up)
    ctx.fill("psi", 0.0)
    for _ in range(AUTOTUNE_ITERS):
        ctx.iterate(want_population=False)
    tuned = ctx.autotune() if not args.no_autotune else None
    active = {k: ctx.get_option(k) for k in ("sweep_tile_xy", "sweep_tile_z", "sweep_reciprocals_active",
                                             "moments_tensor_ltimes", "moments_tensor_lplustimes", "moments_tf32_ltimes",
                                             "moments_tf32_lplustimes", "scattering_tensor_active",
                                             "scattering_block_active")}

    # warm-up (the solve starts from psi = 0, like SteadyStateSolver)
    ctx.fill("psi", 0.0)
    for _ in range(args.warmup):
        ctx.iterate(want_population=False)
    ctx.sync()

    # timed region: K source iterations, CUDA events on the stream the kernels run on
    clocks = ClockSampler(local)
    ctx.reset_timers()
    ctx.set_timing(True)
    launches0 = ctx.launch_count()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ms = timed_steps(ctx, stream, args.steps)
    clk = clocks.stop()
    if world > 1:
        torch.distributed.barrier()
    launches = ctx.launch_count() - launches0
    fam = {f: ctx.kernel_time(f) for f in ("sweep", "ltimes", "lplustimes", "scattering", "source", "population")}
    ctx.set_timing(False)
    part = ctx.population()
    ms = max_over_ranks(ms, world)

    # end to end through the public API with host buffers: upload every generated input from
    # pinned host memory, run a 10-iteration solve (psi reset, populations read back each solve)
    names = [n for n in ("ell", "ell_plus", "sigt_zonal", "data/sigs", "quadrature/xcos", "quadrature/ycos",
                         "quadrature/zcos", "quadrature/w", "quadrature/id", "quadrature/jd", "quadrature/kd", "dx",
                         "dy", "dz", "volume", "zone_to_num_mixelem", "zone_to_mixelem", "mixelem_to_zone",
                         "mixelem_to_material", "mixelem_to_fraction", "moment_to_legendre")]
    host = {}
    if args.no_e2e:
        names = []
    for n in names:
        a = ctx.download(n)
        pinned = torch.empty(a.size, dtype=torch.int32 if a.dtype == np.int32 else torch.float64).pin_memory()
        pinned.numpy()[:] = a
        host[n] = pinned
    h2d = sum(t.numel() * t.element_size() for t in host.values())
    niter = 10
    e2e_times = []
    for rep in range(2 if names else 0):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for n in names:
            ctx.upload(n, host[n].numpy())
        ctx.solve(niter)
        e2e_times.append(time.perf_counter() - t0)
    e2e_value = U * niter / e2e_times[-1] * world if e2e_times else None

    # roofline of the dominant kernel family
    pk = peaks()
    tbytes = 8 if precision == abi.FP64 else 4
    alg = algorithmic(w, tbytes)
    shares = {f: fam[f][0] for f in fam}
    total = sum(shares.values()) or 1.0
    dom = max(shares, key=shares.get)
    dom_ms = fam[dom][0] / args.steps
    flops, nbytes = alg[dom]["flops"], alg[dom]["bytes"]
    if precision == abi.FP64:
        achieved = flops / (dom_ms * 1e-3) / 1e9
        p64, p64_src, p64_clk = fp64_peak(local)
        roof = {"bound": "fp64", "achieved": achieved, "peak": p64, "unit": "GFLOP/s",
                "frac": achieved / p64, "traffic": None, "kernel": dom, "peak_source": p64_src,
                "peak_probe_clocks": p64_clk,
                "hbm": {"achieved": nbytes / (dom_ms * 1e-3) / 1e9, "peak": pk["hbm_gbs"], "unit": "GB/s",
                        "frac": nbytes / (dom_ms * 1e-3) / 1e9 / pk["hbm_gbs"]}}
    else:
        achieved = nbytes / (dom_ms * 1e-3) / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / pk["hbm_gbs"], "traffic": None, "kernel": dom}
    traffic_file = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(traffic_file):
        tr = json.load(open(traffic_file)).get("%s/%s" % (args.precision, dom))
        if tr:
            roof["traffic"] = tr

    line = {
        "metric": "unknowns/s per source iteration", "value": U * world / (ms * 1e-3), "unit": "unknowns/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if precision == abi.FP64 else "f32 (FP64 reductions)",
        "data": "synthetic (seeded generator, no external data)",
        "config": {"workload": WORKLOAD_NAME if not args.zones else WORKLOAD_NAME.replace("64^3", "%d^3" % args.zones),
                   "precision": args.precision, "unknowns": U,
                   "l2": "inputs larger than L2 (psi, rhs 17.2 GB each); no flush",
                   "parallelism": "replicas" if world > 1 else "1 GPU", "autotuned": tuned,
                   "kernels": active},
        "roofline": roof,
        "kernel_ms_per_step": {f: fam[f][0] / args.steps for f in fam},
        "kernel_share": {f: shares[f] / total for f in shares},
        "gpu_launches": launches,
        "clocks": clk,
        "e2e": {"value": e2e_value, "unit": "unknowns/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 8 * niter,
                "step": "upload all inputs from pinned host memory + %d-iteration solve + populations to host" % niter,
                "read_back": "the %d particle counts (the figure of merit); phi and psi stay on the device" % niter},
        "population_after_timed_steps": part,
    }
    mixed = None
    if rank == 0 and world == 1 and precision == abi.FP64 and not args.no_mixed:
        progress("mixed form")
        mixed = mixed_report(args, local, w, ctx, ms)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, dt = cpu_run(CPU_SAMPLE, threads, 1, 2)
        line["cpu_baseline"] = {"value": v, "unit": "unknowns/s", "cores": threads, "kind": "port",
                                "sample": "oracle (OpenMP restatement, equal bit for bit to the reference's own "
                                          "code on its recorded configurations) on the 32^3-zone sample, "
                                          "2 iterations"}
    if rank == 0 and world == 1 and not args.no_adjoint:
        progress("adjoint")
        line["adjoint"] = adjoint_report(local)
    if rank == 0 and world == 1 and not args.no_batch:
        progress("batch")
        line["batch"] = batch_report(local, args.batch_problems)
    if mixed is not None:
        line["mixed"] = mixed
    if rank == 0 and world == 1 and not args.no_parity:
        line["parity"] = parity_report(local, line)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default sweep tile shape")
    ap.add_argument("--option", action="append", default=[], metavar="KEY=VALUE",
                    help="kgb_set_option knob applied before autotuning (repeatable)")
    ap.add_argument("--zones", type=int, default=0, help="override zones per axis (profiling on a smaller case)")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-form comparison")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint gradient report")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-problems report")
    ap.add_argument("--no-parity", action="store_true", help="skip the per-configuration parity report")
    ap.add_argument("--batch-problems", type=int, default=BATCH_PROBLEMS,
                    help="problems in the batched report (profiling on a smaller batch)")
    args = ap.parse_args()
    world, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gpu(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
