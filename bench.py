"""Benchmark: seconds to the permeability tensor of a 256^3 Gaussian-random-field
cell (correlation length 6 voxels, porosity 0.35, seed 1003), three unit load
cases, mixed precision (FP32 FFT / Green multiply / scatter-gather, FP64
Lanczos vectors, inner products and averages), on the GB300.

Output: one JSON line (rank 0).

  value      seconds per permeability tensor, device-resident: the mask and
             the Green table are on the GPU when the timed region starts;
             support extraction + 3 x (RHS, MINRES, recovery) + K.  Timed
             with CUDA events on the library's stream, max over ranks.
  e2e        the same metric through the C ABI with host buffers: fp_create
             (FFT plans + Green precompute) + fp_set_geometry (mask H2D) +
             fp_solve_permeability (K D2H) + fp_destroy, host wall clock.
  roofline   the operator apply (the five FFT passes of one
             scatter -> FFT -> Green -> IFFT -> gather), algorithmic bytes per
             apply / CUDA-event time of the apply, against the measured HBM
             copy bandwidth.
  cpu_baseline  the CPU oracle (plain-C restatement of the reference path, FP64,
             all host threads) on a bounded sample of the same workload,
             extrapolated to the full solve.

``--impl reference`` times the reference's CPU path the same way (the oracle
port; the reference's own build cannot travel to the aarch64 GPU host) and
prints the same metric.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "seconds_to_permeability_tensor_256"
UNIT = "s"
WORKLOAD = "grf256_phi0.35_l6_seed1003_3loadcases"

# Convergence tolerance of the mixed-precision solve.  The K error against the
# FP64 solve (tol 1e-10) is measured and reported in every run.
TOL_MIXED = 1e-7
TOL_FP64 = 1e-10
MAXIT = 20000


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison solve")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--mode", default="solve",
                    choices=["solve", "apply", "batch", "learned", "brinkman", "pradius", "rve",
                             "unet"],
                    help="solve: the headline (seconds to K at 256^3); apply: --reps operator "
                         "applies per precision (for profilers); batch: 64 uneven "
                         "microstructures; brinkman: the C2 Brinkman cell; learned: the "
                         "learned warm start; pradius: K against the Green alias radius; "
                         "rve: RVE-size sweep on the batched engine; unet: U-Net forward "
                         "passes (for profilers)")
    ap.add_argument("--precision", default="mixed,fp64", help="precisions for --mode apply")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--tiling", default="",
                    help="--mode apply / solve: 'auto' (autotune; the default of solve) or "
                         "'tile,tma,x_bulk,x_rows[,lowreg]' (e.g. 16,1,1,4,0)")
    ap.add_argument("--batch-count", type=int, default=64, help="microstructures for --mode batch")
    ap.add_argument("--concurrency", type=int, default=8, help="host threads for --mode batch")
    ap.add_argument("--max-group", type=int, default=16,
                    help="--mode batch: problems of one grid solved as one group")
    ap.add_argument("--pairs", type=int, default=4000, help="training pairs for --mode learned")
    ap.add_argument("--epochs", type=int, default=8, help="training epochs for --mode learned")
    ap.add_argument("--no-512", action="store_true", help="--mode learned: skip the 512^3 cell")
    return ap.parse_args()


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(world, v: float) -> float:
    """Max of a per-rank timing over all ranks (NCCL on GPUs, gloo on CPU)."""
    if world == 1:
        return v
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rank_seed(rank: int) -> int:
    """Weak scaling: each rank solves its own cell, seeded 1003 + rank."""
    return 1003 + rank


def workload_mask(size, seed):
    from fft_method_test_gb300 import geometry as G

    return G.gaussian_field(size, 6.0, 0.35, seed)


# ---------------------------------------------------------------------------
# clocks sampling (nvidia-smi during the timed region)
# ---------------------------------------------------------------------------

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# CUDA events on the library's stream
# ---------------------------------------------------------------------------

class StreamTimer:
    def __init__(self, stream_ptr):
        import torch

        self.torch = torch
        self.stream = torch.cuda.ExternalStream(stream_ptr)

    def event(self):
        e = self.torch.cuda.Event(enable_timing=True)
        e.record(self.stream)
        return e


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def traffic_from_profile():
    """DRAM bytes per operator apply from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "operator_apply_grf256_mixed.md")
    try:
        with open(path) as f:
            for ln in f:
                if ln.startswith("traffic_bytes_per_apply:"):
                    return float(ln.split(":")[1])
    except OSError:
        pass
    return None


def apply_bytes(nh: int, nb: int, precision: str) -> float:
    """Algorithmic HBM bytes of one operator apply with the five-pass fused
    pipeline: 8 sweeps of the 3-component half spectrum, one Green read, the
    compact input read and output write (FP64 vectors) and the int32 support
    index read twice."""
    c = 8 if precision == "mixed" else 16  # complex element
    g = 4 if precision == "mixed" else 8   # Green element
    return 8 * 3 * c * nh + 6 * g * nh + 2 * 3 * 8 * nb + 2 * 4 * nb


# ---------------------------------------------------------------------------
# CPU baseline (oracle restatement): per-unit times and the solve model
# ---------------------------------------------------------------------------

def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc

    return orc


def cpu_units(mask, threads=0, iters=2, ctx=None):
    """Per-unit times of the CPU oracle (the plain-C restatement of the
    reference path, FP64, `threads` OpenMP threads, 0 = all) on this cell:
    setup (support + Green precompute), one operator apply (what the RHS and
    the recovery each cost) and one MINRES iteration (an apply plus the
    Lanczos vector work), the last two timed on the cell itself."""
    orc = _oracle()
    own = ctx is None
    t_setup = None
    if own:
        t0 = time.perf_counter()
        ctx = orc.Restatement().context(mask, threads=threads)
        t_setup = time.perf_counter() - t0
    b = ctx.build_rhs([1.0, 0.0, 0.0])
    x = np.random.default_rng(0).uniform(-1, 1, 3 * ctx.nb)
    t0 = time.perf_counter()
    ctx.operator_apply(x)
    t_apply = time.perf_counter() - t0
    t0 = time.perf_counter()
    ctx.minres(b, 1e-300, 0)
    t_m0 = time.perf_counter() - t0
    t0 = time.perf_counter()
    ctx.minres(b, 1e-300, iters)
    t_iter = max(time.perf_counter() - t0 - t_m0, 0.0) / iters
    if own:
        ctx.close()
    return dict(setup_s=t_setup, apply_s=t_apply, iter_s=t_iter)


def cpu_predict(u, iterations, setups):
    """Seconds to K: `setups` set-ups (the reference recomputes the Green
    tensor for every load case, PermeabilityRunner.cpp:186-203) plus, per
    load case, the RHS apply, its MINRES iterations and the recovery apply."""
    return setups * u["setup_s"] + sum(2 * u["apply_s"] + i * u["iter_s"] for i in iterations)


def cpu_model_check(mask, tol, threads=0):
    """Times one complete CPU permeability solve of `mask` and the model's
    prediction of it from per-unit times taken on the same cell (the oracle
    context computes its set-up once for the three load cases)."""
    orc = _oracle()
    t0 = time.perf_counter()
    ctx = orc.Restatement().context(mask, threads=threads)
    t_setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    _, its = ctx.solve_permeability(tol, MAXIT)
    t_solve = time.perf_counter() - t0
    u = cpu_units(mask, threads, ctx=ctx)
    ctx.close()
    u["setup_s"] = t_setup
    measured = t_setup + t_solve
    predicted = cpu_predict(u, [int(i) for i in its], setups=1)
    return {"grid": list(mask.shape), "tol": tol, "iterations": [int(i) for i in its],
            "measured_s": measured, "predicted_s": predicted,
            "rel_err": (predicted - measured) / measured}


ORACLE_K = os.path.join(ROOT, "tests", "golden", "oracle_k.npz")


def oracle_fixture(name, mask):
    """K and iteration counts of the CPU oracle for a committed cell
    (tests/golden/oracle_k.npz), when the regenerated mask is that cell."""
    import hashlib

    try:
        z = np.load(ORACLE_K)
    except OSError:
        return None
    with z:
        if name + "_K" not in z.files:
            return None
        if hashlib.sha256(np.ascontiguousarray(mask, np.uint8).tobytes()).hexdigest() != str(
                z[name + "_sha256"]):
            return None
        return {"K": z[name + "_K"].copy(), "iterations": [int(i) for i in z[name + "_iters"]],
                "tol": float(z[name + "_tol"])}


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------

def run_ours(args, world, rank, local):
    import ctypes as C

    import torch

    from fft_method_test_gb300 import _capi
    from fft_method_test_gb300.permeability import PermeabilityProblem

    torch.cuda.set_device(local)
    size = args.size
    mask = workload_mask(size, rank_seed(rank))  # weak scaling: one cell per rank
    lib = _capi.load()

    # setup (untimed): problem with Green table + geometry on the device
    t0 = time.perf_counter()
    prob = PermeabilityProblem(mask.shape, precision="mixed")
    t_create = time.perf_counter() - t0
    nb = prob.set_geometry(mask)
    nh = (size // 2 + 1) * size * size
    timer = StreamTimer(lib.fp_stream(prob.handle))
    # FFT tiling picked by timing the apply (cached per grid and precision),
    # the analogue of the reference's FFTW_MEASURE planning; untimed here,
    # its wall time is reported with e2e
    t0 = time.perf_counter()
    if args.tiling and args.tiling != "auto":
        # a fixed tiling (e.g. the tuner's choice of an earlier run), for
        # profilers: the tuner's timings are not meaningful under ncu
        t, tma, xb, xr, lo = (int(v) for v in (args.tiling + ",0").split(",")[:5])
        prob.set_tiling(t, bool(tma), bool(xb), xr, bool(lo))
        tuned = dict(tile=t, tma=bool(tma), x_bulk=bool(xb), x_rows=xr, lowreg=bool(lo), fixed=True)
    else:
        tuned = prob.autotune()
    t_tune = time.perf_counter() - t0

    # FP64 reference solve on the same cell (plain FP64 GPU MINRES)
    K64 = None
    fp64_s = None
    it64 = None
    fp64_same_tol_s = fp64_same_tol_err = it64b = None
    fp64_roof = None
    if not args.no_fp64:
        prob.set_precision("fp64")
        prob.autotune()
        t0 = time.perf_counter()
        K64, st64 = prob.solve_permeability(TOL_FP64, MAXIT)
        fp64_s = time.perf_counter() - t0
        it64 = [s["iterations"] for s in st64]
        # the same tolerance as the mixed solve: the like-for-like FP64 time
        t0 = time.perf_counter()
        K64b, st64b = prob.solve_permeability(TOL_MIXED, MAXIT)
        fp64_same_tol_s = time.perf_counter() - t0
        fp64_same_tol_err = float(np.linalg.norm(K64b - K64) / np.linalg.norm(K64))
        it64b = [s["iterations"] for s in st64b]
        # the FP64 apply against the measured FP64 rate (the bound of the
        # FP64 passes on GB300) and against HBM
        x64 = torch.randn(3 * nb, dtype=torch.float64, device="cuda")
        y64 = torch.empty_like(x64)
        for _ in range(2):
            lib.fp_operator_apply_device(prob.handle, C.c_void_p(x64.data_ptr()),
                                         C.c_void_p(y64.data_ptr()))
        e0 = timer.event()
        for _ in range(5):
            lib.fp_operator_apply_device(prob.handle, C.c_void_p(x64.data_ptr()),
                                         C.c_void_p(y64.data_ptr()))
        e1 = timer.event()
        e1.synchronize()
        t_apply64 = e0.elapsed_time(e1) / 1e3 / 5
        del x64, y64
        rate, rate_ms = C.c_double(0.0), C.c_double(0.0)
        lib.fp_measure_fp64_rate(C.byref(rate), C.byref(rate_ms))
        n = float(size) ** 3
        flops64 = 15.0 * n * np.log2(n) + 36.0 * nh
        hbm_peak, _ = measured_peak_hbm()
        fp64_roof = {"bound": "fp64", "achieved": flops64 / t_apply64 / 1e12,
                     "peak": rate.value, "unit": "TFLOP/s",
                     "frac": flops64 / t_apply64 / 1e12 / rate.value if rate.value > 0 else None,
                     "peak_kind": "measured (fp_measure_fp64_rate, FMA chains)",
                     "flops_per_apply": flops64, "apply_ms": t_apply64 * 1e3,
                     "hbm_frac": apply_bytes(nh, nb, "fp64") / t_apply64 / 1e9 / hbm_peak}
        prob.set_precision("mixed")
        prob.autotune()  # back to the mixed tiling (cached)

    def step(block=True):
        # the three load cases as one lockstep block (fp_solve_permeability_block:
        # the same K and iterations as one by one, one launch per pass for the
        # three fields)
        K, st = prob.solve_permeability(TOL_MIXED, MAXIT, block=block)
        return K, st

    for _ in range(args.warmup):
        K, st = step()
    barrier(world)
    torch.cuda.synchronize()
    times = []
    launches0 = lib.fp_kernel_launch_count()
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            e0 = timer.event()
            K, st = step()
            e1 = timer.event()
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
    torch.cuda.synchronize()
    launches = lib.fp_kernel_launch_count() - launches0
    barrier(world)
    t_step = max_over_ranks(world, float(np.mean(times)))
    its = [s["iterations"] for s in st]
    # the same solve with the load cases one after another (fp_solve_permeability),
    # outside the timed region
    one_by_one = []
    for _ in range(2):
        e0 = timer.event()
        K1, _ = step(block=False)
        e1 = timer.event()
        e1.synchronize()
        one_by_one.append(e0.elapsed_time(e1) / 1e3)
    one_by_one_identical = bool(np.array_equal(K1, K))

    # roofline: operator applies on device-resident vectors
    x = torch.randn(3 * nb, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    torch.cuda.synchronize()
    for _ in range(3):
        lib.fp_operator_apply_device(prob.handle, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()))
    reps = 20
    e0 = timer.event()
    for _ in range(reps):
        lib.fp_operator_apply_device(prob.handle, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()))
    e1 = timer.event()
    e1.synchronize()
    t_apply_full = e0.elapsed_time(e1) / 1e3 / reps
    # the apply as MINRES runs it: the five passes, scatter and gather fused
    # (the input mean comes from the previous vector update, the output mean
    # is removed in the z update), CUDA events on the library's stream
    ms = C.c_double(0.0)
    rc = lib.fp_time_apply(prob.handle, reps, C.byref(ms))
    t_apply = ms.value / 1e3 if rc == 0 else t_apply_full
    peak, peak_kind = measured_peak_hbm()
    bytes_apply = apply_bytes(nh, nb, "mixed")
    achieved = bytes_apply / t_apply / 1e9

    # e2e through the C ABI with host buffers
    mask_c = np.ascontiguousarray(mask, dtype=np.uint8)
    e2e_times = []
    for i in range(max(1, args.steps)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with PermeabilityProblem(mask.shape, precision="mixed") as p2:
            p2.set_geometry(mask_c)
            if tuned.get("fixed"):
                p2.set_tiling(tuned["tile"], tuned["tma"], tuned["x_bulk"], tuned["x_rows"],
                              tuned["lowreg"])
            else:
                p2.autotune()  # the cached tiling of this grid
            K2, _ = p2.solve_permeability(TOL_MIXED, MAXIT, block=True)
        e2e_times.append(time.perf_counter() - t0)
    e2e = max_over_ranks(world, float(np.mean(e2e_times)))

    err = None
    if K64 is not None:
        err = float(np.linalg.norm(K - K64) / np.linalg.norm(K64))
    # the CPU oracle's K of this very cell (committed fixture, tol 1e-7)
    fx = oracle_fixture("grf256", mask) if size == 256 else None
    err_orc = err64_orc = None
    if fx is not None:
        err_orc = float(np.linalg.norm(K - fx["K"]) / np.linalg.norm(fx["K"]))
        if K64 is not None:
            err64_orc = float(np.linalg.norm(K64 - fx["K"]) / np.linalg.norm(fx["K"]))

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        its_cpu = fx["iterations"] if fx else (it64b or its)
        its_from = ("the CPU oracle's own iteration counts at tol %.0e" % fx["tol"] if fx else
                    "the GPU %s solve's iteration counts (oracle fixture absent)"
                    % ("FP64" if it64b else "mixed"))
        u = cpu_units(mask)
        cores = os.cpu_count() or 1
        cpu = {"value": cpu_predict(u, its_cpu, setups=3), "unit": UNIT, "cores": cores,
               "kind": "port",
               "sample": "C restatement of the reference path (FP64, %d threads) at 256^3: set-up "
                         "(support + Green) %.2f s, one apply %.3f s and one MINRES iteration "
                         "(apply + vector work) %.3f s timed on this cell; seconds to K = 3 set-ups "
                         "(the reference recomputes Green per load case) + per load case 2 applies "
                         "+ iterations x iteration time, with %s (%s)"
                         % (cores, u["setup_s"], u["apply_s"], u["iter_s"], its_from, its_cpu)}

    prob.close()
    if rank != 0:
        return
    value = t_step / world if world > 1 else t_step
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32+fp64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "grid": [size, size, size], "load_cases": 3,
                   "precision": "mixed (fp32 FFT/Green/scatter-gather, fp64 Lanczos)",
                   "tol": TOL_MIXED, "support_voxels": nb, "iterations": its,
                   "warm_start": "none", "l2": "working set > L2 (spectral field 3 x (n/2+1) n^2 x 8 B)",
                   "green_precompute_s": t_create, "parallelism": "replicas" if world > 1 else "1gpu",
                   "fft_tiling": tuned, "load_case_schedule": "3-RHS block (fp_solve_permeability_block)"},
        "load_cases_one_by_one": {"seconds": float(np.mean(one_by_one)),
                                  "K_identical_to_block": one_by_one_identical},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(mask.size),
                "d2h_bytes_per_step": 72, "tuning_s": t_tune, "value_with_tuning": e2e + t_tune},
        "K_rel_err_vs_fp64": err, "K_rel_err_vs_oracle": err_orc,
        "fp64_K_rel_err_vs_oracle": err64_orc, "fp64_seconds": fp64_s, "fp64_iterations": it64,
        "fp64_same_tol": {"tol": TOL_MIXED, "seconds": fp64_same_tol_s, "iterations": it64b,
                          "K_rel_err_vs_fp64": fp64_same_tol_err},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic_from_profile(),
                     "kernel": "operator apply as MINRES runs it (5 fused FFT passes)",
                     "peak_kind": peak_kind, "bytes_per_apply": bytes_apply,
                     "apply_ms": t_apply * 1e3,
                     "apply_with_mean_removal_ms": t_apply_full * 1e3,
                     "frac_with_mean_removal": bytes_apply / t_apply_full / 1e9 / peak},
        "fp64_roofline": fp64_roof,
        "cpu_baseline": cpu,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)


def run_reference(args, world, rank, local):
    """The reference's CPU path (the oracle port, FP64, all host threads) on
    the same workload, metric and tolerance as our arm.  One step times the
    per-unit costs on the 256^3 cell (one apply and two MINRES iterations;
    the set-up once); seconds to K follow from the solve model with the CPU
    oracle's own iteration counts at the same tolerance.  The model is
    checked against one complete CPU solve of a 64^3 cell in every run."""
    if rank != 0:
        return
    size = args.size
    mask = workload_mask(size, 1003)
    fx = oracle_fixture("grf256", mask) if size == 256 else None
    if fx is not None:
        its_cpu, its_src = fx["iterations"], "CPU oracle at tol %.0e (tests/golden/oracle_k.npz)" % fx["tol"]
    else:
        its_cpu, its_src = REFERENCE_ITERATIONS_256, "GPU FP64 solve at tol 1e-7 (fixture absent)"
    from fft_method_test_gb300 import geometry as G

    check = cpu_model_check(G.gaussian_field(64, 6.0, 0.35, seed=3064), TOL_MIXED)
    orc = _oracle()
    t0 = time.perf_counter()
    ctx = orc.Restatement().context(mask)
    t_setup = time.perf_counter() - t0
    vals = []
    units = []
    for i in range(args.warmup + args.steps):
        u = cpu_units(mask, ctx=ctx)
        u["setup_s"] = t_setup
        if i >= args.warmup:
            vals.append(cpu_predict(u, its_cpu, setups=3))
            units.append(u)
    ctx.close()
    v = float(np.mean(vals))
    cores = os.cpu_count() or 1
    um = {k: float(np.mean([u[k] for u in units])) for k in ("setup_s", "apply_s", "iter_s")}
    line = {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": v * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": WORKLOAD, "grid": [size, size, size], "load_cases": 3,
                   "tol": TOL_MIXED, "iterations": its_cpu, "iterations_from": its_src},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "C restatement of the reference's CPU path, %d threads: set-up "
                                   "%.2f s once, then per step one apply (%.3f s) and two MINRES "
                                   "iterations (%.3f s each, vector work included) timed at 256^3; "
                                   "seconds to K = 3 set-ups + per load case 2 applies + "
                                   "iterations x iteration time" % (cores, um["setup_s"],
                                                                    um["apply_s"], um["iter_s"])},
        "model_check": check,
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# MINRES iterations of this workload at tol 1e-7 from the GPU FP64 solve
# (which follows the reference's recurrence): 2485 over the three load cases,
# split evenly (the model uses only the sum); used only when the CPU oracle's
# own counts (tests/golden/oracle_k.npz) are absent.
REFERENCE_ITERATIONS_256 = [828, 828, 829]


def run_applies(args):
    """Profiling entry: operator applies on device-resident vectors, nothing else."""
    import ctypes as C

    import torch

    from fft_method_test_gb300.permeability import PermeabilityProblem

    mask = workload_mask(args.size, 1003)
    for prec in args.precision.split(","):
        with PermeabilityProblem(mask.shape, precision=prec) as p:
            nb = p.set_geometry(mask)
            if args.tiling == "auto":
                print(prec, "tiling", p.autotune(), flush=True)
            elif args.tiling:
                t, tma, xb, xr, lo = (int(v) for v in (args.tiling + ",0").split(",")[:5])
                p.set_tiling(t, bool(tma), bool(xb), xr, bool(lo))
            x = torch.randn(3 * nb, dtype=torch.float64, device="cuda")
            y = torch.empty_like(x)
            torch.cuda.synchronize()
            timer = StreamTimer(p.lib.fp_stream(p.handle))
            e0 = timer.event()
            for _ in range(args.reps):
                p.lib.fp_operator_apply_device(p.handle, C.c_void_p(x.data_ptr()),
                                               C.c_void_p(y.data_ptr()))
            e1 = timer.event()
            p.lib.fp_synchronize(p.handle)
            ms = e0.elapsed_time(e1) / max(1, args.reps)
            nh = (args.size // 2 + 1) * args.size * args.size
            gbs = apply_bytes(nh, nb, prec) / (ms * 1e-3) / 1e9
            print("%s apply %.4f ms (%d reps, first ones cold), %.0f GB/s algorithmic"
                  % (prec, ms, args.reps, gbs), flush=True)
    print("applies done", flush=True)


def batch_workload(count: int = 64):
    """64 microstructures, seeds 2000..2063: edge uniform from {48, 64, 80,
    96, 128, 160}, porosity uniform in [0.3, 0.8]; even seeds overlapping
    spheres with radii uniform in [3, 10], odd seeds Gaussian random fields
    with correlation length 6."""
    from fft_method_test_gb300 import geometry as G

    return [G.batch_cell(2000 + i) for i in range(count)]


def run_batch(args):
    """Batched solve of uneven microstructures: voxel-iterations per second
    over the whole batch, in groups of one grid with one launch per pass for
    each group (concurrent groups), one problem per stream (concurrent), and
    one at a time; all autotuned."""
    import torch

    from fft_method_test_gb300 import _capi
    from fft_method_test_gb300.permeability import batch_solve_permeability

    masks = batch_workload(args.batch_count)
    lib = _capi.load()
    vox = np.array([m.size for m in masks], dtype=np.float64)
    out = {}
    Ks = {}
    for label, conc, group in (("grouped", args.concurrency, args.max_group),
                               ("batched", args.concurrency, 1), ("sequential", 1, 1)):
        torch.cuda.synchronize()
        l0 = lib.fp_kernel_launch_count()
        t0 = time.perf_counter()
        K, st, status = batch_solve_permeability(masks, precision="mixed", tol=TOL_MIXED,
                                                 maxit=MAXIT, concurrency=conc, autotune=True,
                                                 max_group=group)
        Ks[label] = K
        dt = time.perf_counter() - t0
        its = np.array([sum(s["iterations"] for s in sp) for sp in st], dtype=np.float64)
        out[label] = dict(seconds=dt, voxel_iterations_per_s=float((vox * its).sum() / dt),
                          iterations=int(its.sum()), launches=int(lib.fp_kernel_launch_count() - l0),
                          all_converged=bool(all(all(s["converged"] for s in sp) for sp in st)),
                          status_ok=bool(all(c == 0 for c in status)))
    line = {"metric": "batch_voxel_iterations_per_s", "value": out["grouped"]["voxel_iterations_per_s"],
            "unit": "voxel*iter/s", "higher_is_better": True, "n_gpus": 1, "dtype": "fp32+fp64",
            "data": "synthetic",
            "config": {"workload": "batch64_edges48-160_spheres_grf_seeds2000-2063",
                       "count": len(masks), "concurrency": args.concurrency,
                       "max_group": args.max_group, "tol": TOL_MIXED,
                       "precision": "mixed", "voxels": int(vox.sum())},
            "grouped": out["grouped"], "batched": out["batched"], "sequential": out["sequential"],
            "K_identical_grouped_vs_sequential": bool(np.array_equal(Ks["grouped"], Ks["sequential"])),
            "speedup_vs_sequential": out["sequential"]["seconds"] / out["grouped"]["seconds"],
            "speedup_batched_vs_sequential": out["sequential"]["seconds"] / out["batched"]["seconds"]}
    print(json.dumps(line), flush=True)


def run_learned(args):
    """The learned warm start as configured: the 4-level U-Net (16 -> 128
    channels, 3x3x3 tcgen05 convolutions) trained on `--pairs` solver-generated
    64^3 pairs (seeds 10000.., spheres and Gaussian fields at porosity
    0.3-0.8), then used as the MINRES initial guess (scaled by the factor that
    minimises the initial residual; zero start when that is not below |b|) on
    the benchmark cell and Gaussian-field cells of porosity 0.25 at 256^3 and
    512^3 (seeds 20000, 20001), mixed precision, tol 1e-7.  Reports training
    cost and loss, and per load case the initial residual, inference time and
    iterations/seconds against the zero start."""
    import torch

    from fft_method_test_gb300 import geometry as G
    from fft_method_test_gb300 import learned as L
    from fft_method_test_gb300.permeability import PermeabilityProblem

    n = 64
    t0 = time.perf_counter()
    pairs = L.make_pairs(args.pairs, n, seed=10000)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    val = L.make_pairs(32, n, seed=10000 + args.pairs)
    net = L.UNetWarmStart(seed=0)
    t0 = time.perf_counter()
    hist = L.train_unet(net, pairs, n, epochs=args.epochs, batch=4, lr=1e-3)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    val_loss = L.evaluate_unet(net, val, n)
    del pairs
    cells = {"grf256_phi0.35_l6_seed1003": workload_mask(256, 1003),
             "grf256_phi0.25_l6_seed20000": G.gaussian_field(256, 6.0, 0.25, seed=20000)}
    if not args.no_512:
        cells["grf512_phi0.25_l6_seed20001"] = G.gaussian_field(512, 6.0, 0.25, seed=20001)
    res = {}
    for name, m in cells.items():
        rows = []
        with PermeabilityProblem(m.shape, precision="mixed") as p:
            p.set_geometry(m)
            p.autotune()
            sup = p.support()
            for d in range(3):
                g = np.zeros(3)
                g[d] = 1.0
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                avg0, s0, _ = p.solve_load_case(g, TOL_MIXED, MAXIT)
                t_zero = time.perf_counter() - t0
                t0 = time.perf_counter()
                x0 = L.predict_guess_unet(net, m, sup, d)
                torch.cuda.synchronize()
                t_inf = time.perf_counter() - t0
                b = p.build_rhs(g)
                ax = p.operator_apply(x0)
                den = float(ax @ ax)
                scale = float(b @ ax) / den if den > 0 else 0.0
                rel0 = float(np.linalg.norm(b - scale * ax) / np.linalg.norm(b))
                use = scale > 0 and rel0 < 1.0
                t_fit = time.perf_counter() - t0 - t_inf
                t0 = time.perf_counter()
                avg1, s1, _ = p.solve_load_case(g, TOL_MIXED, MAXIT, x0=scale * x0 if use else None)
                t_warm = time.perf_counter() - t0
                rows.append({"zero_start": {"iterations": s0["iterations"], "seconds": t_zero},
                             "warm_start": {"iterations": s1["iterations"],
                                            "seconds": t_warm + t_inf + t_fit,
                                            "inference_s": t_inf, "fit_s": t_fit,
                                            "guess_used": bool(use), "initial_rel_residual": rel0},
                             "avg_velocity_rel_diff": float(np.linalg.norm(avg1 - avg0) /
                                                            np.linalg.norm(avg0))})
        res[name] = rows
    line = {"metric": "learned_warm_start", "data": "synthetic", "n_gpus": 1,
            "network": {"levels": 4, "channels": [16, 32, 64, 128], "kernel": "3x3x3",
                        "conv": "tcgen05.mma BF16 -> FP32 (TMEM)",
                        "parameters": int(sum(p["w"].numel() + p["b"].numel()
                                              for p in net.params.values()))},
            "training": {"pairs": args.pairs, "grid": n, "epochs": args.epochs,
                         "data_seconds": t_data, "train_seconds": t_train,
                         "loss_per_epoch": hist, "val_loss": val_loss},
            "tol": TOL_MIXED, "precision": "mixed", "cells": res}
    print(json.dumps(line), flush=True)


def run_unet_forward(args):
    """Profiling entry: the warm-start U-Net's forward pass (tcgen05
    convolutions) on a batch of four 64^3 sphere packings, --reps times."""
    import torch

    from fft_method_test_gb300 import geometry as G
    from fft_method_test_gb300 import learned as L

    net = L.UNetWarmStart(seed=0)
    masks = [G.spheres(64, 5.0, 0.5, seed=k) for k in range(4)]
    m = torch.tensor(np.concatenate([x.ravel() for x in masks]), device="cuda")
    feat = L.features_gpu(m, (m == 0).to(torch.uint8))
    for _ in range(args.reps):
        out, _ = net.forward(feat, (64, 64, 64), 4)
    torch.cuda.synchronize()
    print("unet forward done", float(out.abs().sum()), flush=True)


def run_pradius(args):
    """Convergence of K with the alias radius P of the energy-consistent Green
    sum (the reference fixes P = 2 and leaves the study open,
    GreenOperator.cpp:98): FP64, tol 1e-10, P = 0..4, on the C1 cell (32^3
    spheres r 4, porosity 0.6, seed 1001) and a 64^3 Gaussian field (l 6,
    porosity 0.35, seed 3064).  Reports K and its relative change against
    the largest P."""
    from fft_method_test_gb300 import geometry as G
    from fft_method_test_gb300.permeability import PermeabilityProblem

    cells = {"c1_spheres32": G.spheres(32, 4.0, 0.60, seed=1001),
             "grf64_phi0.35_l6_seed3064": G.gaussian_field(64, 6.0, 0.35, seed=3064)}
    radii = [0, 1, 2, 3, 4]
    out = {}
    for name, m in cells.items():
        Ks = {}
        for pr in radii:
            t0 = time.perf_counter()
            with PermeabilityProblem(m.shape, precision="fp64", p_radius=pr) as p:
                p.set_geometry(m)
                K, st = p.solve_permeability(TOL_FP64, MAXIT)
            Ks[pr] = (K, time.perf_counter() - t0, [s["iterations"] for s in st])
        Kref = Ks[radii[-1]][0]
        out[name] = {str(pr): {"K": np.asarray(K).tolist(), "seconds": t, "iterations": its,
                               "K_rel_diff_vs_P%d" % radii[-1]:
                                   float(np.linalg.norm(K - Kref) / np.linalg.norm(Kref))}
                     for pr, (K, t, its) in Ks.items()}
    print(json.dumps({"metric": "green_alias_radius_study", "data": "synthetic", "n_gpus": 1,
                      "precision": "fp64", "tol": TOL_FP64, "cells": out}), flush=True)


def run_rve(args):
    """RVE-size sweep on the batched engine: Gaussian random fields (l 6,
    porosity 0.35) of edges 32, 48, 64, 96 and 128, eight independent
    realisations per edge (seeds 40000 + 100 * edge + k), solved together by
    fp_batch_solve_permeability (mixed, tol 1e-7).  Reports per edge the mean
    and standard deviation of the diagonal of K and of its mean, the measure
    of how far a cell of that edge is from representative."""
    from fft_method_test_gb300 import geometry as G
    from fft_method_test_gb300.permeability import batch_solve_permeability

    edges = [32, 48, 64, 96, 128]
    reals = 8
    masks, owner = [], []
    for e in edges:
        for k in range(reals):
            masks.append(G.gaussian_field(e, 6.0, 0.35, seed=40000 + 100 * e + k))
            owner.append(e)
    t0 = time.perf_counter()
    K, st, status = batch_solve_permeability(masks, precision="mixed", tol=TOL_MIXED, maxit=MAXIT,
                                             concurrency=args.concurrency, autotune=True,
                                             max_group=args.max_group)
    dt = time.perf_counter() - t0
    res = {}
    for e in edges:
        ks = np.array([np.trace(K[i]) / 3.0 for i in range(len(masks)) if owner[i] == e])
        diag = np.array([np.diag(K[i]) for i in range(len(masks)) if owner[i] == e])
        res[str(e)] = {"realisations": int(len(ks)), "mean_K": float(ks.mean()),
                       "std_K": float(ks.std(ddof=1)), "rel_std": float(ks.std(ddof=1) / ks.mean()),
                       "mean_diag": diag.mean(axis=0).tolist()}
    print(json.dumps({"metric": "rve_size_sweep", "data": "synthetic", "n_gpus": 1,
                      "precision": "mixed", "tol": TOL_MIXED, "seconds": dt,
                      "all_ok": bool(all(c == 0 for c in status)), "edges": res}), flush=True)


def run_brinkman(args):
    """C2: Brinkman penalisation on a 128^3 cell of radius-8 spheres at
    porosity 0.45 (seed 1002), penalty 1e4, viscosity 1, unit force along x.
    Times the reference iteration on the GPU (per-iteration HBM roofline:
    1016 bytes per voxel), the fixed-point solver to tol 1e-8, and the
    reference iteration on the CPU oracle (single thread, as the reference's
    Brinkman builds) on a bounded sample."""
    import torch

    from fft_method_test_gb300 import geometry as G
    from fft_method_test_gb300.permeability import solveBrinkman, solveBrinkmanFixedPoint

    mask = G.spheres(128, 8.0, 0.45, seed=1002)
    ids = G.to_ids(mask)
    n = ids.size
    its = 400  # the reference's default max_iterations
    solveBrinkman(ids, (1.0, 0.0, 0.0), solid_penalty=1e4, tolerance=1e-30, max_iterations=10)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ref = solveBrinkman(ids, (1.0, 0.0, 0.0), solid_penalty=1e4, tolerance=1e-30, max_iterations=its)
    t_ref = time.perf_counter() - t0
    peak, peak_kind = measured_peak_hbm()
    bytes_it = 1016.0 * n
    achieved = bytes_it * its / t_ref / 1e9
    solveBrinkmanFixedPoint(ids, (1.0, 0.0, 0.0), solid_penalty=1e4, tolerance=1e-6)
    t0 = time.perf_counter()
    fpnt = solveBrinkmanFixedPoint(ids, (1.0, 0.0, 0.0), solid_penalty=1e4, tolerance=1e-8)
    t_fp = time.perf_counter() - t0
    U_fp = fpnt["superficialVelocity"]
    cpu = None
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as orc

        R = orc.Restatement()
        k = 5
        t0 = time.perf_counter()
        R.brinkman(ids, tolerance=1e-30, max_iterations=k)
        t_cpu = (time.perf_counter() - t0) / k
        cpu = {"value": t_cpu * its, "unit": "s", "cores": 1, "kind": "port",
               "sample": "C restatement of the reference iteration, %d iterations at 128^3 "
                         "timed (%.3f s each), scaled to %d" % (k, t_cpu, its)}
    # config C2 compares the Brinkman permeability with the variational method
    # on the same geometry (the reference runs both behind one runner,
    # PermeabilityRunner.cpp:250-447 and :451-832): the variational K (FP64,
    # tol 1e-10) and the Brinkman fixed point's K for all three load cases
    from fft_method_test_gb300.permeability import (PermeabilityProblem,
                                                    computePermeabilityTensorFixedPoint)

    t0 = time.perf_counter()
    with PermeabilityProblem(mask.shape, precision="fp64") as pv:
        pv.set_geometry(mask)
        K_var, st_var = pv.solve_permeability(TOL_FP64, MAXIT)
    t_var = time.perf_counter() - t0
    t0 = time.perf_counter()
    K_br, st_br = computePermeabilityTensorFixedPoint(ids, solid_penalty=1e4, tolerance=1e-8)
    t_brk = time.perf_counter() - t0
    # both methods on a plate channel, where the continuum answer is known:
    # solid slab z < 8 in a 64^3 cell, fluid gap g = 56, flow along x;
    # superficial K_xx = porosity * g^2 / 12 (plane Poiseuille flow)
    ch = np.ones((64, 64, 64), np.uint8)
    ch[:8] = 0
    with PermeabilityProblem(ch.shape, precision="fp64") as pv:
        pv.set_geometry(ch)
        K_ch_var, _ = pv.solve_permeability(TOL_FP64, MAXIT)
    K_ch_br, _ = computePermeabilityTensorFixedPoint(G.to_ids(ch), solid_penalty=1e4, tolerance=1e-8)
    channel = {"analytic_Kxx": float(56.0 / 64.0 * 56.0 ** 2 / 12.0),
               "variational_Kxx": float(K_ch_var[0, 0]), "brinkman_Kxx": float(K_ch_br[0, 0])}
    fx = oracle_fixture("c2_128_sph", mask)
    comparison = {
        "plate_channel_64": channel,
        "variational": {"K": np.asarray(K_var).tolist(), "tol": TOL_FP64, "seconds": t_var,
                        "iterations": [s["iterations"] for s in st_var],
                        "K_rel_err_vs_oracle": (float(np.linalg.norm(K_var - fx["K"]) /
                                                      np.linalg.norm(fx["K"])) if fx else None)},
        "brinkman_fixed_point": {"K": np.asarray(K_br).tolist(), "tol": 1e-8, "seconds": t_brk,
                                 "iterations": [s["iterations"] for s in st_br]},
        "K_rel_diff_brinkman_vs_variational": float(np.linalg.norm(np.asarray(K_br) - K_var) /
                                                    np.linalg.norm(K_var)),
    }
    line = {"metric": "brinkman_c2_128", "data": "synthetic", "n_gpus": 1, "dtype": "fp64",
            "config": {"workload": "spheres128_r8_phi0.45_seed1002", "penalty": 1e4, "mu": 1.0,
                       "force": [1.0, 0.0, 0.0]},
            "reference_iteration": {"iterations": its, "seconds": t_ref,
                                    "ms_per_iteration": 1e3 * t_ref / its,
                                    "residual": ref["residual"],
                                    "U_rel_err_vs_fixed_point":
                                        float(abs(ref["superficialVelocity"][0] - U_fp[0]) / abs(U_fp[0])),
                                    "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                                                 "unit": "GB/s", "frac": achieved / peak,
                                                 "peak_kind": peak_kind,
                                                 "bytes_per_iteration": bytes_it}},
            "fixed_point": {"tol": 1e-8, "iterations": fpnt["iterations"], "seconds": t_fp,
                            "converged": bool(fpnt["converged"]), "residual": fpnt["residual"],
                            "U": [float(u) for u in U_fp]},
            "c2_comparison": comparison,
            "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.mode == "brinkman":
        run_brinkman(args)
        return
    if args.mode == "learned":
        run_learned(args)
        return
    if args.mode == "apply":
        run_applies(args)
        return
    if args.mode == "batch":
        run_batch(args)
        return
    if args.mode == "unet":
        run_unet_forward(args)
        return
    if args.mode == "pradius":
        run_pradius(args)
        return
    if args.mode == "rve":
        run_rve(args)
        return
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank, local)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
