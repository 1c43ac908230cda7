"""Benchmark: LM edges linearised per second of a multi-camera local BA.

Workload (one "step"): a full Levenberg-Marquardt local bundle adjustment
(10 iterations; 20 for the large map) of the 30-keyframe x 3-camera window with
20k map points (~150k observations, 5% outliers, Huber sqrt(5.991), first 2
keyframes fixed), solved on one GPU by libmcba in mixed precision.  Metric:
active edges x LM iterations / solve time.  Seeded synthetic data with the
benchmark's shapes and noise model.

  value   device-resident: problem compiled and uploaded once, every step
          restores the initial estimates on the device and solves (CUDA
          events inside the library), L2 flushed between steps.
  e2e     through the C ABI with host buffers: load + optimize (structure
          compilation, H2D, solve, D2H of the solution) per step.
  fp64_plain  the same two measurements of the FP64 plain solve, and the
          final-cost gap and pose error of the mixed solve against it.
  config1  the 10-keyframe window: mixed and FP64 plain rates, the serial
          oracle's rate on it, and the gap.
  cpu_baseline  the oracle (a restatement of the reference's g2o path), one
          thread, on a bounded number of whole solves of the same problem.

--impl reference times the oracle with every host thread on the same
workload (the reference's own code cannot be built here).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

LBA_ITERS = {1: 10, 2: 10, 5: 20}  # LM iterations per configuration
FP64_NOMINAL_GFLOPS = 1250.0  # FP64 rate of the part (nominal)
PIVOT_CHAIN_CYCLES = 300      # dependent FP64 FMA (64) + reciprocal seed and cubic Newton step (~237)


def clk_mhz_nominal() -> float:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f).get("sm_max_mhz", 2070.0))
    except (OSError, ValueError):
        return 2070.0


def metric_name(pr, iters: int) -> str:
    return (f"LM edges linearised/s (local BA, {pr.n_poses} KF x 3 cams, {pr.n_points // 1000}k points, "
            f"{iters} LM iterations)")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mcba", choices=["mcba", "reference"])
    ap.add_argument("--config", type=int, default=2, choices=[1, 2, 4, 5])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--iters", type=int, default=None,
                    help="LM iterations per solve (default: 10 for configs 1 and 2, 20 for config 5)")
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the FP64-plain comparison and the config-1 block")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--windows", type=int, default=64,
                    help="local-BA windows of --config 4 (64 is the benchmark; fewer for a profiler capture)")
    ap.add_argument("--workload", default="ba", choices=["ba", "knn", "project", "stereo"],
                    help="ba: the local-BA solve (default); knn: brute-force Hamming k=2 matching; "
                         "project: map-point projection + windowed match over a batch of objects; "
                         "stereo: stereo matching of a batch of rectified frames")
    ap.add_argument("--frames", type=int, default=256, help="stereo frames for --workload stereo")
    ap.add_argument("--objects", type=int, default=512, help="objects (frame cameras) for --workload project")
    ap.add_argument("--knn-n", type=int, default=32768, help="query and train descriptors for --workload knn")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


# ------------------------------------------------------------------ clocks --
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for i, n in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------- roofline --
def algorithmic_bytes_linearize(st: dict, precision: str) -> int:
    """Compulsory bytes of one linearisation launch.

    Per active edge: the streamed record (pose, point, camera, flags,
    information, Huber threshold, u v) = 28 B in FP32 / 40 B in FP64, plus the
    6x3 Hpl block it must produce for the Schur step (72 B / 144 B).
    Per free point: read X (12 B / 24 B) and write Hll + b_l (9 values).
    Per free pose: read the pose (48 B / 96 B) and write Hpp + b_p (27 values)."""
    w = 4 if precision == "mixed" else 8
    rec = 28 if precision == "mixed" else 40
    E, Lf, Kf = st["n_active_edges"], st["n_free_points"], st["n_free_poses"]
    return E * (rec + 18 * w) + Lf * (3 * w + 9 * w) + Kf * (12 * w + 27 * w)


def read_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def fp64_peak(local: int):
    """(GFLOP/s, source) of FP64 FMA: measured on the device by the library's
    saturating FMA kernel, else the part's nominal rate."""
    import ctypes

    from mcvslam_gb300 import _native

    g = ctypes.c_double(0.0)
    if _native.lib().mcba_fp64_fma_rate(local, ctypes.byref(g)) == 0 and g.value > 0:
        return g.value, "measured (mcba_fp64_fma_rate: saturating FMA kernel, CUDA events, best of 5)"
    return FP64_NOMINAL_GFLOPS, "nominal FP64 rate of the part"


def read_traffic(kernel: str):
    """Per-launch DRAM bytes of `kernel` recorded from an ncu capture in profiles/."""
    prof = os.path.join(ROOT, "profiles")
    try:
        names = sorted(os.listdir(prof))
    except OSError:
        return None
    for n in names:
        if not n.endswith(".md"):
            continue
        with open(os.path.join(prof, n)) as f:
            for line in f:
                if line.startswith(f"traffic_bytes_per_launch[{kernel}]:"):
                    try:
                        return int(float(line.split(":", 1)[1].strip()))
                    except ValueError:
                        return None
    return None


# --------------------------------------------------------------------- arms --
def iters_of(args) -> int:
    return args.iters if args.iters is not None else LBA_ITERS.get(args.config, 10)


def cpu_baseline(pr, seconds: float, iters: int) -> dict:
    from oracle import oracle

    t0 = time.perf_counter()
    runs, edges = 0, 0
    while True:
        r = oracle.optimize(pr, iters, n_threads=1, log_cap=1)
        runs += 1
        edges += r["n_active_edges"] * max(r["iterations_done"], 0)
        if time.perf_counter() - t0 >= seconds or runs >= 50:
            break
    dt = time.perf_counter() - t0
    return {"value": edges / dt, "unit": "edges/s", "cores": 1, "kind": "port",
            "sample": f"{runs} whole {iters}-iteration solves of the same problem, serial oracle, {dt:.1f} s"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from mcvslam_gb300 import synth
    from oracle import oracle

    pr = synth.config(args.config)
    iters = iters_of(args)
    threads = os.cpu_count() or 1
    times, edges = [], 0
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        r = oracle.optimize(pr, iters, n_threads=threads, log_cap=1)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
            edges = r["n_active_edges"] * max(r["iterations_done"], 0)
    ms = 1e3 * statistics.mean(times)
    value = edges / (ms / 1e3)
    line = {
        "impl": "reference", "metric": metric_name(pr, iters), "value": value, "unit": "edges/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
        "config": {"workload": pr.name, "edges": pr.n_edges, "keyframes": pr.n_poses, "points": pr.n_points,
                   "lm_iterations": iters, "solver": "oracle restatement of g2o LM + Schur, OpenMP"},
        "cpu_baseline": {"value": value, "unit": "edges/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} whole solves after {args.warmup} warm-up"},
        "e2e": {"value": value, "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_knn_reference(args):
    """The oracle's KnnMatch (the reference's cv::parallel_for_ loop restated,
    OpenMP over every host thread) on a bounded sample of the same sets."""
    rank, _, _ = dist_env()
    if rank != 0:
        return
    from mcvslam_gb300 import synth
    from oracle import oracle

    n = args.knn_n
    q, t = synth.descriptors(n, n, 5100)
    threads = os.cpu_count() or 1
    rows = n
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        oracle.knn_hamming(q, t, n_threads=threads)
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    ms = 1e3 * statistics.mean(times)
    value = rows * float(n) / (ms / 1e3)
    line = {
        "impl": "reference", "metric": "Hamming k=2 descriptor pairs compared/s", "value": value,
        "unit": "pairs/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic ORB-like descriptors", "config": {"workload": f"knn_hamming_{n}x{n}"},
        "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": threads, "kind": "port",
                         "sample": f"each step the whole {n} x {n} match"},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _device_leg(ba, pr, precision, iters, steps, warmup, flush, local):
    """Device-resident solves (problem uploaded once, initial estimates
    restored on the device each step, L2 flushed before each): the open
    solver, per-step device ms, kernel launches and the last stats."""
    import torch

    s = ba.Solver(precision=precision, device=local, use_graph=True)
    s.load(pr)
    s.prepare()
    for _ in range(warmup):
        s.solve_prepared(iters)
    step_ms, launches, st = [], 0, None
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        st = s.solve_prepared(iters)
        step_ms.append(st["ms_total"])
        launches += st["kernel_launches"]
    return s, step_ms, launches, st


def _e2e_leg(ba, pr, precision, iters, steps, warmup, local, world):
    """The same solve through the C ABI with host buffers: create, load
    (structure compilation, H2D), optimize, read the estimates back, destroy."""
    import torch

    e2e_ms, h2d, d2h, st2 = [], 0, 0, None
    for i in range(warmup + steps):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        with ba.Solver(precision=precision, device=local) as s2:
            s2.load(pr)
            st2 = s2.optimize(iters)
            s2.state()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t1
        if i >= warmup:
            e2e_ms.append(1e3 * dt)
            h2d, d2h = st2["h2d_bytes"], st2["d2h_bytes"]
    return {"value": world * st2["edges_linearized"] / (statistics.mean(e2e_ms) / 1e3), "unit": "edges/s",
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "ms_per_step": statistics.mean(e2e_ms)}


def _fp64_cost(ba, pr, qt, X, local) -> float:
    """activeRobustChi2 of the estimates (qt, X), evaluated in FP64."""
    with ba.Solver(precision="fp64", device=local) as s:
        s.load(pr)
        s.set_state(qt, X)
        return s.optimize(0)["initial_chi2"]


def _rot_err(qa, qb) -> float:
    va, vb = np.asarray(qa[:3]), np.asarray(qb[:3])
    w = qa[3] * qb[3] + va @ vb
    v = qb[3] * va - qa[3] * vb - np.cross(va, vb)
    return float(2 * np.arctan2(np.linalg.norm(v), abs(w)))


def _gap(ba, pr, mixed_state, plain_state, plain_chi, local) -> dict:
    """Final-cost gap of the mixed solve (its estimates costed in FP64) and its
    largest pose difference, against the FP64 plain solve."""
    chi_m = _fp64_cost(ba, pr, mixed_state[0], mixed_state[1], local)
    qm, qp = mixed_state[0], plain_state[0]
    return {"final_cost_rel": (chi_m - plain_chi) / plain_chi, "bound": 1e-6,
            "within_bound": bool(abs(chi_m - plain_chi) <= 1e-6 * plain_chi),
            "mixed_final_chi2_fp64": chi_m, "fp64_final_chi2": plain_chi,
            "max_pose_err_m": float(np.abs(qm[:, 4:] - qp[:, 4:]).max()),
            "max_pose_err_rad": max(_rot_err(qm[k, :4], qp[k, :4]) for k in range(len(qm)))}


def _compare(ba, pr, iters, steps, warmup, flush, local, world, with_e2e: bool) -> dict:
    """Mixed and FP64 plain on one problem: device-resident rates, optional
    end-to-end rates, and the gap."""
    out = {}
    states = {}
    for prec in ("mixed", "fp64"):
        s, ms, _, st = _device_leg(ba, pr, prec, iters, steps, warmup, flush, local)
        s.fetch_state()
        states[prec] = s.state()
        s.close()
        m = statistics.mean(ms)
        out[prec] = {"value": world * st["edges_linearized"] / (m / 1e3), "unit": "edges/s", "ms_per_step": m,
                     "final_chi2": st["final_chi2"], "lm_trials": st["trials"]}
        if with_e2e:
            out[prec]["e2e"] = _e2e_leg(ba, pr, prec, iters, steps, warmup, local, world)
    out["gap"] = _gap(ba, pr, states["mixed"], states["fp64"], out["fp64"]["final_chi2"], local)
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    return out


def run_mcba(args):
    import torch

    from mcvslam_gb300 import _native, ba, synth

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist_mod

        dist_mod.init_process_group("nccl")
        dist = dist_mod

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    pr = synth.config(args.config)
    iters = iters_of(args)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    # device-resident leg: the LM loop runs as one CUDA graph per solve
    s = ba.Solver(precision=args.precision, device=local, use_graph=True)
    s.load(pr)
    s.prepare()
    for _ in range(args.warmup):
        s.solve_prepared(iters)
    clocks = ClockSampler(local)
    step_ms, launches, stats = [], 0, []
    barrier()
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        st = s.solve_prepared(iters)
        step_ms.append(st["ms_total"])
        launches += st["kernel_launches"]
        stats.append(st)
    barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    st0 = stats[-1]
    s.fetch_state()
    state_main = s.state()
    edges_per_step = st0["edges_linearized"]
    ms = statistics.mean(step_ms)
    t_max = ms
    if dist:
        tt = torch.tensor([ms], device=f"cuda:{local}")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_max = float(tt.item())
    value = world * edges_per_step / (t_max / 1e3)

    # per-kernel durations: the same solves with CUDA events around every
    # phase (host-driven loop, events on the library's stream), L2 flushed
    sp = ba.Solver(precision=args.precision, device=local, profile=True)
    sp.load(pr)
    sp.prepare()
    sp.solve_prepared(iters)
    phase_ms = np.zeros(8)
    phase_n = np.zeros(8, np.int64)
    prof_ms = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        stp = sp.solve_prepared(iters)
        phase_ms += np.array(stp["ms_phase"])
        phase_n += np.array(stp["n_phase"])
        prof_ms.append(stp["ms_total"])
    sp.close()
    phases = {n: {"ms_total": float(phase_ms[i]), "launches": int(phase_n[i]),
                  "ms_per_launch": float(phase_ms[i] / phase_n[i]) if phase_n[i] else None}
              for i, n in enumerate(_native.PHASES)}
    lin_ms = phase_ms[0] / max(phase_n[0], 1)
    alg = algorithmic_bytes_linearize(st0, args.precision)
    peak, peak_kind = read_peaks()
    achieved = alg / (lin_ms / 1e3) / 1e9
    roofline = {"kernel": "k_linearize", "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind, "traffic": read_traffic("k_linearize"),
                "algorithmic_bytes_per_launch": alg, "ms_per_launch": lin_ms,
                "timing": "CUDA events around each launch, host-driven profiled pass of the same solves"}
    # the kernel with the largest share of the solve: the FP64 factorisation of
    # the reduced camera system -- for up to 384 unknowns one cluster kernel
    # bound by its pivot chain, beyond that the tiled kernels, bound by FP64
    # throughput and their panel chain
    chol_ms = phase_ms[5] / max(phase_n[5], 1)
    nred = 6 * int(st0["n_free_poses"])
    flops = nred ** 3 / 3.0 + 4.0 * nred ** 2
    fp64_gf, fp64_src = fp64_peak(local)
    achieved_gf = flops / (chol_ms / 1e3) / 1e9
    roofline_dominant = {
        "kernel": "k_ldlt_cluster" if nred <= 384 else "k_tchol_* (tiled)",
        "bound": "fp64 latency chain" if nred <= 384 else "fp64 throughput + panel chain",
        "achieved": achieved_gf, "peak": fp64_gf, "unit": "GFLOP/s", "frac": achieved_gf / fp64_gf,
        "peak_source": fp64_src, "ms_per_launch": chol_ms, "n": nred,
        "share_of_solve": float(phase_ms[5] / max(sum(prof_ms), 1e-9)),
        "throughput_floor_ms": flops / (fp64_gf * 1e9) * 1e3,
        "chain_floor_us": nred * PIVOT_CHAIN_CYCLES / clk_mhz_nominal() if nred else None,
        "note": "n^3/3 + 4 n^2 flops per solve (factorisation and both substitutions); the chain floor is one "
                f"dependent FP64 pivot step (about {PIVOT_CHAIN_CYCLES} cycles) per unknown"}

    # end-to-end leg through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        e2e = _e2e_leg(ba, pr, args.precision, iters, args.steps, args.warmup, local, world)

    # FP64 plain beside the mixed solve: rates and the final-cost gap
    fp64_plain = gap = cfg1 = None
    if args.precision == "mixed" and not args.no_compare:
        sf, fms, _, stf = _device_leg(ba, pr, "fp64", iters, args.steps, args.warmup, flush, local)
        sf.fetch_state()
        state_fp64 = sf.state()
        sf.close()
        fm = statistics.mean(fms)
        fp64_plain = {"value": world * stf["edges_linearized"] / (fm / 1e3), "unit": "edges/s", "ms_per_step": fm,
                      "final_chi2": stf["final_chi2"], "lm_trials": stf["trials"]}
        if not args.no_e2e:
            fp64_plain["e2e"] = _e2e_leg(ba, pr, "fp64", iters, args.steps, args.warmup, local, world)
        gap = _gap(ba, pr, state_main, state_fp64, stf["final_chi2"], local)
        if args.config == 2:
            # the 10-keyframe window the speed-up target is stated on
            p1 = synth.config(1)
            cfg1 = {"workload": p1.name, "edges": p1.n_edges, "lm_iterations": LBA_ITERS[1]}
            cfg1.update(_compare(ba, p1, LBA_ITERS[1], args.steps, args.warmup, flush, local, world, True))

    cpu = cpu1 = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(pr, args.cpu_seconds, iters)
        if cfg1 is not None:
            cpu1 = cpu_baseline(synth.config(1), min(args.cpu_seconds, 4.0), LBA_ITERS[1])
            cfg1["cpu_baseline"] = cpu1
            cfg1["mixed_over_cpu_serial"] = cfg1["mixed"]["value"] / cpu1["value"]
            cfg1["mixed_e2e_over_cpu_serial"] = cfg1["mixed"]["e2e"]["value"] / cpu1["value"]
            cfg1["target"] = ("mixed >= 20x the serial CPU restatement's edges/s, faster than FP64 plain, "
                              "final-cost gap <= 1e-6")

    if rank == 0:
        line = {
            "metric": metric_name(pr, iters), "value": value, "unit": "edges/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if args.precision == "mixed" else "f64",
            "data": "synthetic (seeded generator with the benchmark's shapes and noise model)",
            "config": {"workload": pr.name, "edges": pr.n_edges, "active_edges": st0["n_active_edges"],
                       "keyframes": pr.n_poses, "free_keyframes": st0["n_free_poses"], "points": pr.n_points,
                       "lm_iterations": iters, "precision": args.precision,
                       "l2": "flushed (256 MB write) before every step",
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "ba_solve_ms": ms, "final_chi2": st0["final_chi2"], "lm_trials": st0["trials"]},
            "e2e": e2e, "fp64_plain": fp64_plain, "precision_gap": gap, "config1": cfg1,
            "cpu_baseline": cpu, "roofline": roofline, "roofline_dominant": roofline_dominant,
            "phases": phases,
            "profiled_ms_per_step": statistics.mean(prof_ms),
            "clocks": clk, "gpu_launches": int(launches), "wall_s_timed_region": wall,
        }
        print(json.dumps(line), flush=True)
    s.close()
    if dist:
        dist.destroy_process_group()


def run_config4(args):
    """Batched uneven problems: 64 local-BA windows (U(5,40) keyframes, U(50,300)
    points per keyframe) in one persistent launch (clusters take windows from
    a device work queue; CTAs per window chosen by the autotuner), and 256
    pose-only frames (U(500,6000) observations, 10% outliers, 4 rounds x 10
    iterations) in one persistent launch; mixed precision.

    value = window edges linearised / s (device-resident persistent launch);
    e2e = the same through the C ABI with host buffers (64 loads, one batch
    compile/upload, one launch, 64 read-backs); the same windows as branches
    of one CUDA graph beside it; the per-window final-cost gap of the mixed
    solves against FP64 solves of the same windows; the roofline of
    k_linearize over the windows from host-driven profiled passes."""
    import torch

    from mcvslam_gb300 import ba, synth

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    iters = LBA_ITERS[2]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    wins = synth.window_batch(args.windows)
    rng = np.random.default_rng(4100)
    frames = [synth.pose_only(int(rng.integers(500, 6001)), seed=4200 + i) for i in range(256)]
    clocks = ClockSampler(local)
    with ba.LocalBABatch(wins, precision="mixed", device=local) as b:
        # the same windows as branches of one CUDA graph
        for _ in range(args.warmup):
            b.solve(iters)
        gms = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            gstats, ms = b.solve(iters)
            gms.append(ms)
        graph_final = [st["final_chi2"] for st in gstats]
        for _ in range(args.warmup):
            b.solve(iters, persistent=True)
        wms, edges, launches = [], 0, 0
        clocks.start()
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            stats, ms = b.solve(iters, persistent=True)
            wms.append(ms)
            edges = sum(st["edges_linearized"] for st in stats)
            launches += sum(st["kernel_launches"] for st in stats)
        cluster_ctas = b.cluster_ctas
        for _ in range(args.warmup):
            ba.batch_pose_only(frames, "mixed", rounds=4, iterations=10, device=local)
        pms = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            pms.append(ba.batch_pose_only(frames, "mixed", rounds=4, iterations=10, device=local)["ms_device"])
        clk = clocks.stop()
        mixed_states = b.states()
        mixed_final = [st["final_chi2"] for st in stats]
    w_ms, p_ms = statistics.mean(wms), statistics.mean(pms)
    # the same windows in FP64 plain, and the FP64 cost of each mixed result
    with ba.LocalBABatch(wins, precision="fp64", device=local) as bf:
        bf.solve(iters, persistent=True)
        fstats, f_ms = bf.solve(iters, persistent=True)
    gaps = []
    for pr, (qt, X), fs in zip(wins, mixed_states, fstats):
        chi_m = _fp64_cost(ba, pr, qt, X, local)
        gaps.append((chi_m - fs["final_chi2"]) / fs["final_chi2"])
    gaps = np.array(gaps)
    # end to end through the C ABI with host buffers
    e2e_ms, pe2e_ms = [], []
    for i in range(0 if args.no_e2e else args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with ba.LocalBABatch(wins, precision="mixed", device=local) as b2:
            b2.solve(iters, persistent=True)
            b2.states()
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e_ms.append(1e3 * (time.perf_counter() - t0))
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        ba.batch_pose_only(frames, "mixed", rounds=4, iterations=10, device=local)
        if i >= args.warmup:
            pe2e_ms.append(1e3 * (time.perf_counter() - t0))
    h2d = int(sum(28 * w.n_edges + 28 * w.n_poses + 12 * w.n_points for w in wins))
    d2h = int(sum(56 * w.n_poses + 24 * w.n_points for w in wins))
    # k_linearize over every window: host-driven profiled passes
    lin_ms, alg = 0.0, 0
    for pr in wins:
        sp = ba.Solver(precision="mixed", device=local, profile=True)
        sp.load(pr)
        sp.prepare()
        sp.solve_prepared(iters)
        stp = sp.solve_prepared(iters)
        sp.close()
        if stp["n_phase"][0]:
            lin_ms += stp["ms_phase"][0] / stp["n_phase"][0]
            alg += algorithmic_bytes_linearize(stp, "mixed")
    peak, peak_kind = read_peaks()
    lin_gbs = alg / (lin_ms / 1e3) / 1e9 if lin_ms > 0 else None
    roofline = {"kernel": "k_linearize (64 windows, one launch each)", "bound": "hbm", "achieved": lin_gbs,
                "peak": peak, "unit": "GB/s", "frac": lin_gbs / peak if lin_gbs else None, "peak_source": peak_kind,
                "traffic": None, "algorithmic_bytes": alg, "ms_sum_of_launches": lin_ms,
                "note": "sum of the 64 windows' algorithmic bytes over the sum of their event-timed launches; "
                        "small windows are launch- and latency-bound"}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import oracle

        t0 = time.perf_counter()
        e_cpu = 0
        for pr in wins[:3]:
            r = oracle.optimize(pr, iters, n_threads=1, log_cap=1)
            e_cpu += r["n_active_edges"] * max(r["iterations_done"], 0)
        dt = time.perf_counter() - t0
        t1 = time.perf_counter()
        for fr in frames[:16]:
            oracle.pose_optimization(fr, rounds=4, iters=10, chi2_thr=5.991)
        dtp = time.perf_counter() - t1
        cpu = {"value": e_cpu / dt, "unit": "edges/s", "cores": 1, "kind": "port",
               "sample": f"3 of the 64 windows, {iters} LM iterations each, serial oracle, {dt:.1f} s",
               "pose_only_frames_per_s": 16 / dtp,
               "pose_only_sample": f"16 of the 256 frames, 4 rounds x 10 iterations, serial oracle, {dtp:.1f} s"}
    if rank == 0:
        line = {
            "metric": "LM edges linearised/s, 64 local-BA windows in one persistent launch",
            "value": edges / (w_ms / 1e3),
            "unit": "edges/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": w_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded generator with the benchmark's shapes and noise model)",
            "config": {"workload": "config4_batched", "windows": len(wins), "cluster_ctas_per_window": cluster_ctas,
                       "graph_branches": {"ms_per_step": statistics.mean(gms),
                                          "value": edges / (statistics.mean(gms) / 1e3),
                                          "same_final_chi2_as_persistent": graph_final == mixed_final},
                       "window_edges": int(sum(w.n_edges for w in wins)), "lm_iterations": iters,
                       "pose_only_frames": len(frames), "pose_only_edges": int(sum(f.n_edges for f in frames)),
                       "pose_only_ms": p_ms, "pose_only_frames_per_s": len(frames) / (p_ms / 1e3),
                       "l2": "flushed (256 MB write) before every step"},
            "e2e": None if not e2e_ms else {
                "value": edges / (statistics.mean(e2e_ms) / 1e3), "unit": "edges/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": statistics.mean(e2e_ms),
                "pose_only_ms": statistics.mean(pe2e_ms),
                "pose_only_frames_per_s": len(frames) / (statistics.mean(pe2e_ms) / 1e3)},
            "fp64_plain": {"ms_per_step": f_ms, "value": sum(s["edges_linearized"] for s in fstats) / (f_ms / 1e3)},
            "precision_gap": {"per_window_final_cost_rel": [float(g) for g in gaps],
                              "max_abs": float(np.abs(gaps).max()), "bound": 1e-6,
                              "windows_within_bound": int((np.abs(gaps) <= 1e-6).sum()),
                              "mixed_final_chi2": mixed_final},
            "roofline": roofline, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": int(launches),
        }
        print(json.dumps(line), flush=True)


# Integer-pipe ceiling of the carry-save Hamming distance: per pair 5 POPC at
# 16 per SM per clock and about 20 ALU operations (8 XOR, 6 carry-save LOP3,
# 3 adds, 3 min/max) at 64 per SM per clock -- both 3.2 pairs per SM per clock.
KNN_PAIRS_PER_SM_CLK = 3.2


def run_knn(args):
    """Matcher::KnnMatch (k = 2) of args.knn_n query descriptors against as many
    train descriptors (32 bytes each), the brute-force distance kernel behind
    stereo, projection and BoW matching.  value = descriptor pairs compared
    per second with both sets resident; e2e = the same through the host-buffer
    C entry (copies in and out inside the timed region)."""
    import ctypes

    import torch

    from mcvslam_gb300 import _native as N
    from mcvslam_gb300 import matcher, synth

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    n = args.knn_n
    q, t = synth.descriptors(n, n, 5100)
    dq, dt = torch.from_numpy(q).cuda(), torch.from_numpy(t).cuda()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        matcher.knn_hamming_device(dq, dt)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for a, b in ev:
        flush.zero_()
        a.record(stream)
        idx, dist, keep = matcher.knn_hamming_device(dq, dt)
        b.record(stream)
    torch.cuda.synchronize()
    ms = statistics.mean(a.elapsed_time(b) for a, b in ev)
    # e2e through the host entry: H2D of both sets, kernels, D2H of idx/dist/keep
    for _ in range(2):
        matcher.knn_hamming(q, t)
    e2e_ms = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        matcher.knn_hamming(q, t)
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    clk = clocks.stop()
    # small case: one frame's stereo match (2000 x 2000), latency per call
    qs, ts = synth.descriptors(2000, 2000, 5200)
    dqs, dts = torch.from_numpy(qs).cuda(), torch.from_numpy(ts).cuda()
    for _ in range(3):
        matcher.knn_hamming_device(dqs, dts)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(100):
        matcher.knn_hamming_device(dqs, dts)
    b.record(stream)
    torch.cuda.synchronize()
    small_us = 1e3 * a.elapsed_time(b) / 100
    pairs = float(n) * n
    launches = 2 * args.steps
    line = None
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            from oracle import oracle

            threads = os.cpu_count() or 1
            runs, t0 = 0, time.perf_counter()
            while True:
                oracle.knn_hamming(q, t, n_threads=threads)
                runs += 1
                if time.perf_counter() - t0 >= 3.0 or runs >= 20:
                    break
            dtc = time.perf_counter() - t0
            cpu = {"value": runs * pairs / dtc, "unit": "pairs/s", "cores": threads, "kind": "port",
                   "sample": f"{runs} whole {n} x {n} matches, OpenMP oracle, {dtc:.1f} s"}
        sm_mhz = clk.get("sm_mhz") or 1920.0
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        peak = sms * sm_mhz * 1e6 * KNN_PAIRS_PER_SM_CLK
        achieved = pairs / (ms / 1e3)
        line = {
            "metric": "Hamming k=2 descriptor pairs compared/s", "value": achieved, "unit": "pairs/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic ORB-like descriptors (60% re-observations with 0-40 flipped bits)",
            "config": {"workload": f"knn_hamming_{n}x{n}", "queries": n, "train": n,
                       "stereo_2000x2000_us": small_us, "l2": "flushed (256 MB write) before every step"},
            "e2e": {"value": pairs / (statistics.mean(e2e_ms) / 1e3), "unit": "pairs/s",
                    "h2d_bytes_per_step": 64 * n, "d2h_bytes_per_step": 17 * n},
            "roofline": {"bound": "int-pipes (ALU + population count)", "achieved": achieved, "peak": peak,
                         "unit": "pairs/s", "frac": achieved / peak, "traffic": None,
                         "peak_basis": f"{KNN_PAIRS_PER_SM_CLK} pairs/SM/clk (5 POPC at 16/clk, ~20 ALU ops at "
                                       f"64/clk per pair) x {sms} SMs x {sm_mhz:.0f} MHz (median sampled); "
                                       "nominal pipe rates, not measured"},
            "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches,
        }
        print(json.dumps(line), flush=True)


PROJ_KP, PROJ_MP = 2000, 3000  # keypoints and local-map points per object


def run_project(args):
    """Object::ProjectBunchMapPoints over args.objects objects (one camera of
    one frame each: 2000 keypoints, 3000 local map points, radius 10 px x ORB
    scale), all in one call.  value = map points projected and matched per
    second with the batch resident; e2e = the host-buffer C entry (validation,
    copies in and out inside the timed region)."""
    import torch

    from mcvslam_gb300 import matcher, synth

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    b = synth.projection_batch(args.objects, PROJ_KP, PROJ_MP, 6100)
    nm = int(b.mp_begin[-1])
    db = matcher.DeviceProjectionBatch(b, device=local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        db.run()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for a, e in ev:
        db.reset()
        flush.zero_()
        a.record(stream)
        db.run(reset=False)
        e.record(stream)
    torch.cuda.synchronize()
    ms = statistics.mean(a.elapsed_time(e) for a, e in ev)
    matched = int(db.count.sum().item())
    for _ in range(2):
        matcher.project_match(b, device=local)
    e2e_ms = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        matcher.project_match(b, device=local)
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    clk = clocks.stop()
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle

        sub = synth.projection_batch(32, PROJ_KP, PROJ_MP, 6100)
        runs, t0 = 0, time.perf_counter()
        while True:
            oracle.project_match(sub, n_threads=1)
            runs += 1
            if time.perf_counter() - t0 >= 3.0 or runs >= 20:
                break
        dtc = time.perf_counter() - t0
        cpu = {"value": runs * 32 * PROJ_MP / dtc, "unit": "map points/s", "cores": 1, "kind": "port",
               "sample": f"{runs} x 32 objects of the same shape, serial oracle, {dtc:.1f} s"}
    nk = int(b.kp_begin[-1])
    h2d = (b.obj_Rt.nbytes + b.obj_K.nbytes + b.obj_size.nbytes + b.obj_radius.nbytes + b.obj_scale.nbytes +
           b.kp_begin.nbytes + b.kp_xy.nbytes + b.kp_desc.nbytes + b.mp_begin.nbytes + b.mp_X.nbytes +
           b.mp_desc.nbytes + b.mp_level.nbytes + b.mp_id.nbytes + b.mp_prev_kp.nbytes + b.kp_bind.nbytes)
    # compulsory bytes of one call: every keypoint's position, descriptor and
    # binding (read + write), every map point's position, descriptor, level,
    # id and previous binding, its match written back
    alg = nk * (8 + 32 + 8) + nm * (12 + 32 + 12 + 4)
    peak, peak_kind = read_peaks()
    achieved = alg / (ms / 1e3) / 1e9
    line = {
        "metric": "map points projected + window-matched/s", "value": nm / (ms / 1e3), "unit": "map points/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64+u32",
        "data": "synthetic: reference-rig cameras, 70% of map points observed with perturbed descriptors, clutter",
        "config": {"workload": f"project_match_{args.objects}x{PROJ_MP}", "objects": args.objects,
                   "keypoints": nk, "map_points": nm, "matched": matched, "radius_px": 10.0,
                   "l2": "flushed (256 MB write) before every step"},
        "e2e": {"value": nm / (statistics.mean(e2e_ms) / 1e3), "unit": "map points/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": 4 * nk + 4 * nm + 4 * args.objects},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "peak_kind": peak_kind,
                     "note": "all three kernels of one call over the compulsory bytes; the search is bound by "
                             "dependent L2 gathers, not by DRAM bandwidth"},
        "cpu_baseline": cpu, "clocks": clk, "gpu_launches": 3 * args.steps,
    }
    print(json.dumps(line), flush=True)


def run_project_reference(args):
    """The oracle's ProjectBunchMapPoints over the same batch, objects spread
    over every host thread."""
    rank, _, _ = dist_env()
    if rank != 0:
        return
    from mcvslam_gb300 import synth
    from oracle import oracle

    b = synth.projection_batch(args.objects, PROJ_KP, PROJ_MP, 6100)
    threads = os.cpu_count() or 1
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        oracle.project_match(b, n_threads=threads)
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    ms = 1e3 * statistics.mean(times)
    nm = int(b.mp_begin[-1])
    value = nm / (ms / 1e3)
    line = {
        "impl": "reference", "metric": "map points projected + window-matched/s", "value": value,
        "unit": "map points/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64+u32",
        "data": "synthetic", "config": {"workload": f"project_match_{args.objects}x{PROJ_MP}"},
        "cpu_baseline": {"value": value, "unit": "map points/s", "cores": threads, "kind": "port",
                         "sample": "each step the whole batch, objects over OpenMP threads"},
        "e2e": {"value": value, "unit": "map points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


STEREO_LEFT, STEREO_CLUTTER = 1500, 500  # left keypoints and unmatched right keypoints per frame


def run_stereo(args):
    """Frame::ComputeStereoMatch over args.frames rectified 512 x 512 frames
    (8-level pyramids, 1500 left keypoints, ~1200 true right counterparts plus
    500 clutter keypoints each), all in one call.  value = frames per second
    with the batch resident; e2e = the host-buffer C entry (pyramids and
    keypoints copied in, u_right/depth copied out)."""
    import torch

    from mcvslam_gb300 import matcher, synth

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    sb = synth.stereo_batch(args.frames, STEREO_LEFT, STEREO_CLUTTER, 7100)
    db = matcher.DeviceStereoBatch(sb, device=local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        db.run()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for a, e in ev:
        flush.zero_()
        a.record(stream)
        u, _ = db.run()
        e.record(stream)
    torch.cuda.synchronize()
    ms = statistics.mean(a.elapsed_time(e) for a, e in ev)
    matched = int((u >= 0).sum().item())
    for _ in range(2):
        matcher.stereo_match(sb, device=local)
    e2e_ms = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        matcher.stereo_match(sb, device=local)
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    clk = clocks.stop()
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle

        sub = synth.stereo_batch(16, STEREO_LEFT, STEREO_CLUTTER, 7100)
        runs, t0 = 0, time.perf_counter()
        while True:
            oracle.stereo_match(sub, n_threads=1)
            runs += 1
            if time.perf_counter() - t0 >= 3.0 or runs >= 20:
                break
        dtc = time.perf_counter() - t0
        cpu = {"value": runs * 16 / dtc, "unit": "frames/s", "cores": 1, "kind": "port",
               "sample": f"{runs} x 16 frames of the same shape, serial oracle, {dtc:.1f} s"}
    nl, nr = int(sb.left_begin[-1]), int(sb.right_begin[-1])
    pyr = 2 * args.frames * sb.pyr_bytes
    h2d = pyr + sb.left_xy.nbytes + sb.left_oct.nbytes + sb.left_desc.nbytes + sb.right_xy.nbytes + \
        sb.right_oct.nbytes + sb.right_desc.nbytes + 8 * (args.frames + 1)
    # compulsory bytes: keypoints and descriptors once, the 11 x 21 patch
    # bytes of the matched keypoints, the outputs
    alg = nl * (8 + 4 + 32 + 8) + nr * (8 + 4 + 32) + matched * (11 * 11 + 11 * 21)
    peak, peak_kind = read_peaks()
    achieved = alg / (ms / 1e3) / 1e9
    line = {
        "metric": "stereo frames matched/s", "value": args.frames / (ms / 1e3), "unit": "frames/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8+i32+f32",
        "data": "synthetic: textured pyramids, right = left shifted by the frame disparity + noise",
        "config": {"workload": f"stereo_match_{args.frames}x{STEREO_LEFT}", "frames": args.frames,
                   "left_keypoints": nl, "right_keypoints": nr, "kept_matches": matched, "image": "512x512x8 levels",
                   "l2": "flushed (256 MB write) before every step"},
        "e2e": {"value": args.frames / (statistics.mean(e2e_ms) / 1e3), "unit": "frames/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": 8 * nl},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "peak_kind": peak_kind,
                     "note": "three kernels of one call over the compulsory bytes; latency-bound gathers"},
        "cpu_baseline": cpu, "clocks": clk, "gpu_launches": 3 * args.steps,
    }
    print(json.dumps(line), flush=True)


def run_stereo_reference(args):
    """The oracle's ComputeStereoMatch over the same frames, spread over every host thread."""
    rank, _, _ = dist_env()
    if rank != 0:
        return
    from mcvslam_gb300 import synth
    from oracle import oracle

    sb = synth.stereo_batch(args.frames, STEREO_LEFT, STEREO_CLUTTER, 7100)
    threads = os.cpu_count() or 1
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        oracle.stereo_match(sb, n_threads=threads)
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    ms = 1e3 * statistics.mean(times)
    value = args.frames / (ms / 1e3)
    line = {
        "impl": "reference", "metric": "stereo frames matched/s", "value": value, "unit": "frames/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8+i32+f32",
        "data": "synthetic", "config": {"workload": f"stereo_match_{args.frames}x{STEREO_LEFT}"},
        "cpu_baseline": {"value": value, "unit": "frames/s", "cores": threads, "kind": "port",
                         "sample": "each step the whole batch, frames over OpenMP threads"},
        "e2e": {"value": value, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.workload == "stereo":
        if args.impl == "reference":
            run_stereo_reference(args)
        else:
            run_stereo(args)
    elif args.workload == "project":
        if args.impl == "reference":
            run_project_reference(args)
        else:
            run_project(args)
    elif args.workload == "knn":
        if args.impl == "reference":
            run_knn_reference(args)
        else:
            run_knn(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.config == 4:
        run_config4(args)
    else:
        run_mcba(args)


if __name__ == "__main__":
    main()
