"""Benchmark of the hot path: control-point solve + batched evaluation.

Workload (one step): a 3D cubic non-periodic table on a 256^3 mesh of FP64
values f = exp(-r^2) cos(4x) + N(0, 1e-3^2) on [-1, 1]^3 is built (control
points solved on the GPU), then evaluated for value and d/dx at 1e8 query
points -- half uniform in the cube, half Gaussian (sigma 0.05) around 8
random centres in [-0.8, 0.8]^3, interleaved at random. Synthetic, seeded
data of the shapes the reference's workload description names.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line. `value` is points evaluated per second over whole steps
(solve + evaluation) with inputs resident in HBM; `e2e` is the same metric
through the C-ABI host-buffer path (values and coordinates copied from
pinned host memory, results copied back, inside the timed region).
Multi-GPU runs are independent replicas (the path does not exchange data):
`value` sums the points of all ranks over the slowest rank's time.
`--impl reference` times the reference's own CPU code on the host cores:
its headers compiled with g++ -O3 INTP_MULTITHREAD (oracle/_ref, from the
reference install staged under baseline/_ref), over whole steps.

Besides the headline, the line carries the 2D cubic 64^2 workload
(`plain_2d_64`) and the periodic order-7 512^2 workload (`periodic_o7_512`),
each timed on the GPU in both forms and on the reference CPU path, with the
GPU's error against the reference outputs, and the headline's error against
the reference on the CPU baseline's sample (`max_rel_err_vs_reference`).
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

SEED = 20261203 + 1
N_MESH = 256
N_PTS = 100_000_000
DERIVS = [[0, 0, 0], [1, 0, 0]]
PEAKS_PATH = os.path.join(HERE, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
METRIC = "3D cubic evals/s & solve ms, FP32-mixed vs FP64 at stated err; serve p99"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--npts", type=int, default=N_PTS)
    ap.add_argument("--mesh", type=int, default=N_MESH)
    ap.add_argument("--refine", type=int, default=-1,
                    help="mixed solve: 0 = plain FP32 solve, else (default -1) the double-word solve")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64-form comparison")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer measurement")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-tables workload")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving-loop workload")
    ap.add_argument("--no-configs", action="store_true", help="skip the 2D cubic and periodic order-7 workloads")
    ap.add_argument("--cpu-sample", type=int, default=20_000_000,
                    help="points of the CPU baseline's bounded sample (our arm)")
    ap.add_argument("--ref-seconds", type=float, default=90.0,
                    help="reference arm: time budget of the timed whole steps")
    ap.add_argument("--serve-seconds", type=float, default=6.0)
    ap.add_argument("--serve-slots", type=int, default=8, help="server slots (concurrent work units)")
    ap.add_argument("--serve-runs", type=int, default=3,
                    help="runs of the same seeded arrival trace (p99 of each is reported)")
    ap.add_argument("--batched-tables", type=int, default=4096)
    ap.add_argument("--batched-only", action="store_true",
                    help="run only the batched-tables workload (profiling)")
    ap.add_argument("--serve-only", action="store_true", help="run only the serving-loop workload")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------
def make_values_np(n, rng):
    g = np.linspace(-1.0, 1.0, n)
    x = g[:, None, None]
    y = g[None, :, None]
    z = g[None, None, :]
    f = np.exp(-(x * x + y * y + z * z)) * np.cos(4 * x)
    return f + rng.normal(0.0, 1e-3, (n, n, n))


def make_points_np(npts, rng):
    pts = rng.uniform(-1.0, 1.0, (npts, 3))
    centres = rng.uniform(-0.8, 0.8, (8, 3))
    clustered = rng.random(npts) < 0.5
    idx = np.nonzero(clustered)[0]
    which = rng.integers(0, 8, idx.size)
    g = centres[which] + rng.normal(0.0, 0.05, (idx.size, 3))
    for _ in range(8):  # resample points that left the domain
        bad = np.any(np.abs(g) > 1.0, axis=1)
        if not bad.any():
            break
        g[bad] = centres[which[bad]] + rng.normal(0.0, 0.05, (int(bad.sum()), 3))
    pts[idx] = np.clip(g, -1.0, 1.0)
    return pts


def make_workload_gpu(torch, n, npts, seed):
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    g = torch.linspace(-1.0, 1.0, n, device="cuda", dtype=torch.float64)
    x = g[:, None, None]
    y = g[None, :, None]
    z = g[None, None, :]
    vals = torch.exp(-(x * x + y * y + z * z)) * torch.cos(4 * x)
    vals = vals + 1e-3 * torch.randn((n, n, n), device="cuda", dtype=torch.float64, generator=gen)
    pts = torch.rand((npts, 3), device="cuda", dtype=torch.float64, generator=gen) * 2 - 1
    centres = torch.rand((8, 3), device="cuda", dtype=torch.float64, generator=gen) * 1.6 - 0.8
    clustered = torch.rand(npts, device="cuda", generator=gen) < 0.5
    idx = torch.nonzero(clustered).squeeze(1)
    which = torch.randint(0, 8, (idx.numel(),), device="cuda", generator=gen)
    gpts = centres[which] + 0.05 * torch.randn((idx.numel(), 3), device="cuda", dtype=torch.float64,
                                               generator=gen)
    for _ in range(8):
        bad = (gpts.abs() > 1.0).any(dim=1)
        nb = int(bad.sum())
        if nb == 0:
            break
        gpts[bad] = centres[which[bad]] + 0.05 * torch.randn((nb, 3), device="cuda",
                                                             dtype=torch.float64, generator=gen)
    pts[idx] = gpts.clamp(-1.0, 1.0)
    return vals.contiguous(), pts.contiguous()


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for name, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU baseline: the reference's own code on the host cores
# ---------------------------------------------------------------------------
def _reference_available():
    from oracle import reference
    return all(reference.available(lay) for lay in reference.LAYOUTS)


def _pick_layout(order, periodic, vals, lo, hi, pts, derivs, threads, npts_step):
    """Builds the reference in both control-point layouts (INTP_CELL_LAYOUT
    and plain) and keeps the one with the shorter projected step (build +
    npts_step evaluations at the rate measured on `pts`)."""
    from oracle import reference
    best = None
    for layout in reference.LAYOUTS:
        f = reference.RefFunction(order, periodic, vals, lo, hi, layout=layout)
        t0 = time.perf_counter()
        f.outputs(pts, derivs, nthreads=threads)
        rate = pts.shape[0] / (time.perf_counter() - t0)
        step = f.build_seconds + npts_step / rate
        if best is None or step < best[0]:
            best = (step, layout, f, rate)
        else:
            del f
    return best[1], best[2]


def cpu_baseline(npts_step, mesh_n, sample_pts):
    """Times the reference CPU path on a bounded sample of the 3D cubic
    workload, all host threads: the reference headers (INTP_MULTITHREAD, the
    faster of the cell and plain layouts) when oracle/_ref is built, else the
    C restatement. The sample is the full 256^3 build plus `sample_pts` of the
    npts_step points (value and d/dx); the step time is build + npts_step /
    measured rate. Returns (result, (values, points, outputs)) so that the GPU
    outputs can be checked against the same reference outputs."""
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(SEED)
    vals = make_values_np(mesh_n, rng)
    pts = make_points_np(sample_pts, rng)
    lo, hi = [-1.0] * 3, [1.0] * 3
    if _reference_available():
        layout, f = _pick_layout(3, [False] * 3, vals, lo, hi, pts[:1_000_000], DERIVS, threads, npts_step)
        build_s = f.build_seconds
        t0 = time.perf_counter()
        out = f.outputs(pts, DERIVS, nthreads=threads)
        eval_s = time.perf_counter() - t0
        kind = "reference"
        what = "reference headers (g++ -O3 INTP_MULTITHREAD, %s layout)" % layout
    else:
        from oracle import oracle
        s = oracle.Spline(3, 3, [0, 0, 0], [mesh_n] * 3, lo, hi)
        t0 = time.perf_counter()
        s.interpolate(vals, nthreads=threads)
        t1 = time.perf_counter()
        out = s.derivative(pts, DERIVS, nthreads=threads)
        build_s, eval_s = t1 - t0, time.perf_counter() - t1
        kind = "port"
        what = "C restatement of the reference (reference build unavailable)"
    rate = sample_pts / eval_s
    res = {
        "value": npts_step / (build_s + npts_step / rate),
        "unit": "points/s",
        "cores": threads,
        "kind": kind,
        "sample": "%s: full %d^3 build + %d of %d points (value and d/dx); step time = build + %d / measured rate"
                  % (what, mesh_n, sample_pts, npts_step, npts_step),
        "build_ms": build_s * 1e3,
        "eval_points_per_s": rate,
    }
    return res, (vals, pts, out)


def max_rel_err(got, want):
    """max |got - want| / max |want| per output column."""
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    return [float(np.max(np.abs(got[:, k] - want[:, k])) / max(np.max(np.abs(want[:, k])), 1e-300))
            for k in range(want.shape[1])]


# ---------------------------------------------------------------------------
# configs 1 and 4: plain 2D cubic 64^2, periodic order 7 512^2
# ---------------------------------------------------------------------------
CFG1 = dict(name="plain_2d_64", order=3, n=(64, 64), periodic=[False, False], lo=[0.0, 0.0], hi=[1.0, 2.0],
            npts=100_000, derivs=[[0, 0]], seed=20261203 + 0,
            workload="2D order 3 non-periodic 64x64 on [0,1]x[0,2], z = sin(3x)cos(2y) + N(0,0.01^2); "
                     "1e5 uniform points, value")
CFG4 = dict(name="periodic_o7_512", order=7, n=(512, 512), periodic=[True, True], lo=[0.0, 0.0],
            hi=[2 * np.pi, 2 * np.pi], npts=10_000_000, derivs=[[1, 0], [0, 1], [2, 0], [1, 1], [0, 2]],
            seed=20261203 + 3,
            workload="2D order 7 periodic x periodic 512x512, sum of 16 random sinusoids (wavenumbers 1-20); "
                     "cyclic-band solve, then 1e7 uniform points: d/dx, d/dy, d2/dx2, d2/dxdy, d2/dy2")


def config_inputs(cfg):
    rng = np.random.default_rng(cfg["seed"])
    n0, n1 = cfg["n"]
    if cfg["name"] == "plain_2d_64":
        x = np.linspace(0.0, 1.0, n0)
        y = np.linspace(0.0, 2.0, n1)
        vals = np.sin(3 * x)[:, None] * np.cos(2 * y)[None, :] + rng.normal(0.0, 0.01, (n0, n1))
    else:
        g0 = np.arange(n0) * (2 * np.pi / n0)  # one period over the axis range
        g1 = np.arange(n1) * (2 * np.pi / n1)
        X, Y = np.meshgrid(g0, g1, indexing="ij")
        vals = np.zeros((n0, n1))
        for _ in range(16):
            kx, ky = rng.integers(1, 21, 2)
            vals += np.sin(kx * X + ky * Y + rng.uniform(0, 2 * np.pi))
    pts = rng.uniform(cfg["lo"], cfg["hi"], (cfg["npts"], 2))
    return vals, pts


def config_cpu(cfg, vals, pts):
    """The reference CPU path on one whole step of a config (build + every
    point), all host threads; returns (timing, outputs)."""
    threads = os.cpu_count() or 1
    if _reference_available():
        sel = pts[:min(pts.shape[0], 200_000)]
        layout, f = _pick_layout(cfg["order"], cfg["periodic"], vals, cfg["lo"], cfg["hi"], sel, cfg["derivs"],
                                 threads, pts.shape[0])
        # the selection built both layouts; the timed step builds again
        from oracle import reference
        f = reference.RefFunction(cfg["order"], cfg["periodic"], vals, cfg["lo"], cfg["hi"], layout=layout)
        build_s = f.build_seconds
        t0 = time.perf_counter()
        out = f.outputs(pts, cfg["derivs"], nthreads=threads)
        eval_s = time.perf_counter() - t0
        kind = "reference (%s layout)" % layout
    else:
        from oracle import oracle
        s = oracle.Spline(2, cfg["order"], cfg["periodic"], list(cfg["n"]), cfg["lo"], cfg["hi"])
        t0 = time.perf_counter()
        s.interpolate(vals, nthreads=threads)
        t1 = time.perf_counter()
        out = s.derivative(pts, cfg["derivs"], nthreads=threads)
        build_s, eval_s = t1 - t0, time.perf_counter() - t1
        kind = "port"
    npts = pts.shape[0]
    return {"points_per_s": npts / (build_s + eval_s), "build_ms": build_s * 1e3, "eval_ms": eval_s * 1e3,
            "cores": threads, "kind": kind, "steps": 1}, out


def config_gpu(cfg, vals, pts, torch, precision, steps=10, warmup=3):
    """One step = the table's build (control-point solve) + evaluation of
    every point; CUDA events on the launching stream, inputs in HBM."""
    import bsplineinterpolation_gb300 as bi
    r0, r1 = (cfg["lo"][0], cfg["hi"][0]), (cfg["lo"][1], cfg["hi"][1])
    v = torch.tensor(vals, device="cuda")
    p = torch.tensor(pts, device="cuda")
    f = bi.InterpolationFunction(cfg["order"], cfg["periodic"], v, r0, r1, precision=precision)
    out = torch.empty((pts.shape[0], len(cfg["derivs"])), device="cuda",
                      dtype=torch.float32 if precision == "mixed" else torch.float64)
    tpl = f._template
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        tpl._solve(v)
        f.evaluate(p, derivs=cfg["derivs"], out=out)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for e0, e1, e2 in ev:
        e0.record(stream)
        tpl._solve(v)
        e1.record(stream)
        f.evaluate(p, derivs=cfg["derivs"], out=out)
        e2.record(stream)
    torch.cuda.synchronize()
    total = ev[0][0].elapsed_time(ev[-1][2]) / steps
    res = {"points_per_s": pts.shape[0] / (total / 1e3),
           "build_ms": float(np.median([a.elapsed_time(b) for a, b, _ in ev])),
           "eval_ms": float(np.median([b.elapsed_time(c) for _, b, c in ev])),
           "steps": steps, "warmup": warmup}
    return res, out.double().cpu().numpy()


def run_config(cfg, torch):
    vals, pts = config_inputs(cfg)
    cpu, want = config_cpu(cfg, vals, pts)
    res = {"workload": cfg["workload"], "points": int(pts.shape[0]), "cpu_reference": cpu}
    for prec in ("fp64", "mixed"):
        g, got = config_gpu(cfg, vals, pts, torch, prec)
        errs = max_rel_err(got, want)
        g["max_rel_err_vs_reference"] = dict(zip([str(d) for d in cfg["derivs"]], errs))
        res[prec] = g
    res["norm"] = "max|err| / max|reference| per output, over every point"
    return res


# ---------------------------------------------------------------------------
# our implementation
# ---------------------------------------------------------------------------
def peak_hbm():
    try:
        with open(PEAKS_PATH) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def profile_traffic():
    """Per-launch DRAM bytes of the eval kernel from the committed ncu summary."""
    path = os.path.join(HERE, "profiles", "eval_binned_3d_cubic_256.md")
    try:
        with open(path) as fh:
            for line in fh:
                if line.startswith("traffic_bytes_per_launch_full:"):
                    return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def make_reduce_max(dist, torch, device):
    """Max over ranks of a float (all-reduce on `device`)."""
    def reduce_max(v):
        t = torch.tensor([float(v)], device=device, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return reduce_max


def replica_throughput(local_ms, pts_per_rank, steps, world, reduce_max=None):
    """Whole-job points/s of `world` independent replicas: every rank's points
    over the slowest rank's time. Returns (value, max_ms)."""
    t_max = reduce_max(local_ms) if reduce_max else float(local_ms)
    return pts_per_rank * world * steps / (t_max / 1e3), t_max


def run_ours(args, rank, world):
    import torch
    import bsplineinterpolation_gb300 as bi
    from bsplineinterpolation_gb300 import _lib

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    lib = _lib.load()
    n, npts = args.mesh, args.npts
    vals, pts = make_workload_gpu(torch, n, npts, SEED + rank)
    K = len(DERIVS)
    stream = torch.cuda.current_stream()

    def build(precision):
        return bi.InterpolationFunction(3, [False] * 3, vals, (-1.0, 1.0), (-1.0, 1.0), (-1.0, 1.0),
                                        precision=precision, refine_steps=args.refine)

    def timed_steps(f, steps, warmup, out):
        tpl = f._template
        for _ in range(warmup):
            tpl._solve(vals)
            f.evaluate(pts, derivs=DERIVS, out=out)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
               torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        c0 = lib.intp_launch_count()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for e0, e1, e2 in ev:
            e0.record(stream)
            tpl._solve(vals)
            e1.record(stream)
            f.evaluate(pts, derivs=DERIVS, out=out)
            e2.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        launches = lib.intp_launch_count() - c0
        solve = [a.elapsed_time(b) for a, b, _ in ev]
        evalt = [b.elapsed_time(c) for _, b, c in ev]
        total = ev[0][0].elapsed_time(ev[-1][2])
        return total, solve, evalt, wall, launches

    prec = args.precision
    f = build(prec)
    out = torch.empty((npts, K), device="cuda",
                      dtype=torch.float32 if prec == "mixed" else torch.float64)
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    total_ms, solve_ms, eval_ms, wall, launches = timed_steps(f, args.steps, args.warmup, out)
    clock_info = clocks.stop()
    value, t_max = replica_throughput(total_ms, npts, args.steps, world,
                                      make_reduce_max(dist, torch, "cuda") if dist else None)
    result = {
        "metric": METRIC,
        "value": value,
        "unit": "points/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t_max / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32" if prec == "mixed" else "f64",
        "data": "synthetic (seeded; shapes and distributions of the 3D cubic workload)",
        "config": {"workload": "3D cubic 256^3 build + 1e8 queries value+d/dx"
                   if (n == N_MESH and npts == N_PTS) else "3D cubic %d^3 build + %d queries" % (n, npts),
                   "mesh": [n, n, n], "order": 3, "periodic": [False] * 3, "queries": npts,
                   "outputs": ["value", "d/dx"], "precision": prec, "refine_steps": args.refine,
                   "l2": "inputs larger than L2 (values %.0f MB, coordinates %.0f MB)"
                         % (n ** 3 * 8 / 1e6, npts * 24 / 1e6),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "solve_ms": float(np.median(solve_ms)),
        "eval_ms": float(np.median(eval_ms)),
        "gpu_launches": int(launches),
    }
    # roofline of the dominant kernel (evaluation): algorithmic bytes per launch
    out_b = 4 if prec == "mixed" else 8
    table_b = n ** 3 * out_b
    alg_bytes = npts * (24 + K * out_b) + table_b
    peak, peak_kind = peak_hbm()
    ach = alg_bytes / (float(np.median(eval_ms)) / 1e3) / 1e9
    traffic = profile_traffic()
    result["roofline"] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                          "frac": ach / peak, "traffic": traffic,
                          "kernel": "evaluation", "algorithmic_bytes": alg_bytes,
                          "peak_source": peak_kind}
    # the solve: the separable algorithm's own traffic, one read and one write
    # of the mesh per axis pass (3 passes) in the working precision (FP64, or
    # the mixed form's double-words: 8 bytes per value either way)
    solve_b = 8
    solve_bytes = 3 * 2 * n ** 3 * solve_b
    solve_ms_med = float(np.median(solve_ms))
    sach = solve_bytes / (solve_ms_med / 1e3) / 1e9
    result["solve_roofline"] = {"bound": "hbm", "achieved": sach, "peak": peak, "unit": "GB/s",
                                "frac": sach / peak, "algorithmic_bytes": solve_bytes,
                                "compulsory_bytes": 2 * n ** 3 * out_b, "peak_source": peak_kind,
                                "note": "algorithmic bytes: 3 passes x (read + write) x N^3 x %d B (the mixed "
                                        "build solves in double-word arithmetic, 8 B per value)" % solve_b}
    if clock_info:
        result["clocks"] = clock_info

    if rank == 0 and not args.no_fp64 and prec == "mixed":
        f64 = build("fp64")
        out64 = torch.empty((npts, K), device="cuda", dtype=torch.float64)
        tot64, s64, e64, _, _ = timed_steps(f64, 2, 1, out64)
        ref64 = out64
        errs = []
        for k in range(K):
            den = ref64[:, k].abs().max().item()
            errs.append((out[:, k].double() - ref64[:, k]).abs().max().item() / den)
        s64m = float(np.median(s64))
        result["fp64_plain"] = {"points_per_s": npts * 2 / (tot64 / 1e3),
                                "solve_ms": s64m, "eval_ms": float(np.median(e64)),
                                "solve_roofline_frac": 3 * 2 * n ** 3 * 8 / (s64m / 1e3) / 1e9 / peak}
        result["mixed_max_rel_err_vs_fp64"] = {"value": errs[0], "d/dx": errs[1],
                                               "norm": "max|err| / max|fp64| over all queries"}
        del f64, out64

    if rank == 0 and not args.no_e2e:
        result["e2e"] = e2e(args, f, vals, pts, lib, torch)
    if rank == 0 and not args.no_batched:
        result["batched"] = run_batched(args, torch)
    if rank == 0 and not args.no_serve:
        result["serving"] = run_serving(args, torch)
    if rank == 0 and not args.no_cpu:
        base, check = cpu_baseline(npts, n, min(npts, args.cpu_sample))
        result["cpu_baseline"] = base
        result["max_rel_err_vs_reference"] = oracle_check(check, torch)
    if rank == 0 and not args.no_configs:
        result["plain_2d_64"] = run_config(CFG1, torch)
        result["periodic_o7_512"] = run_config(CFG4, torch)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return result


def oracle_check(check, torch):
    """Both GPU forms built from the CPU sample's value mesh and evaluated at
    its points, against the reference CPU path's outputs on them."""
    import bsplineinterpolation_gb300 as bi
    vals, pts, want = check
    v = torch.tensor(vals, device="cuda")
    p = torch.tensor(pts, device="cuda")
    res = {"points": int(pts.shape[0]), "norm": "max|err| / max|reference| per output over the sample"}
    for prec in ("fp64", "mixed"):
        f = bi.InterpolationFunction(3, [False] * 3, v, (-1.0, 1.0), (-1.0, 1.0), (-1.0, 1.0), precision=prec)
        got = f.evaluate(p, derivs=DERIVS).double().cpu().numpy()
        errs = max_rel_err(got, want)
        res[prec] = {"value": errs[0], "d/dx": errs[1]}
        del f
    return res


def e2e(args, f, vals, pts, lib, torch):
    """Same metric through the C-ABI with host buffers: the step copies the
    values and coordinates from pinned host memory, solves, evaluates and
    copies the results back."""
    import bsplineinterpolation_gb300 as bi
    npts = pts.shape[0]
    K = len(DERIVS)
    # page-locked host buffers from the library's own host allocator
    # (intp_host_alloc); the inputs are copied in before the timed region
    hv = torch.from_numpy(bi.host_empty(tuple(vals.shape), np.float64))
    hv.copy_(vals)
    hp = torch.from_numpy(bi.host_empty(tuple(pts.shape), np.float64))
    hp.copy_(pts)
    od = _out_dtype(args)
    ho = torch.from_numpy(bi.host_empty((npts, K), np.float32 if od == 1 else np.float64))
    karr = np.ascontiguousarray(DERIVS, np.int32)
    h = f._h
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def step():
        st = lib.intp_table_interpolate(h, C.c_void_p(hv.data_ptr()), 0, stream)
        if st != 0:
            raise RuntimeError(lib.intp_last_error())
        st = lib.intp_eval_host(h, C.c_void_p(hp.data_ptr()), npts, karr.ctypes.data, K,
                                C.c_void_p(ho.data_ptr()), od, stream)
        if st != 0:
            raise RuntimeError(lib.intp_last_error())

    for _ in range(max(1, min(args.warmup, 2))):
        step()
    torch.cuda.synchronize()
    # at least 10 steps (about 0.15 s): the device slows down for tens of ms
    # about every 0.5 s on these hosts, and a window of a few steps that
    # meets one such slowdown misstates the rate by up to 3x
    steps = max(10, args.steps)
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    return {"value": npts * steps / dt, "unit": "points/s",
            "h2d_bytes_per_step": int(hv.numel() * 8 + hp.numel() * 8),
            "d2h_bytes_per_step": int(ho.numel() * ho.element_size()),
            "ms_per_step": dt / steps * 1e3}


def _out_dtype(args):
    return 1 if args.precision == "mixed" else 0


# ---------------------------------------------------------------------------
# batched tables: 4096 independent tables in one batch
# ---------------------------------------------------------------------------
def _fourier(rng, n, periodic):
    L = n if periodic else n - 1
    x = np.arange(n, dtype=np.float64)
    f = np.zeros(n)
    for k in range(1, 9):
        f += rng.normal(0.0, 1.0 / k) * np.cos(2 * np.pi * k * x / L + rng.uniform(0, 2 * np.pi))
    return f


def make_batched_workload(ntables, seed):
    """Half 1D tables with N ~ U[16, 4096], half 2D with sides ~ U[16, 256];
    orders 3 or 5; 30% periodic (all axes); 8-mode random Fourier values with
    amplitudes ~ N(0, 1/k^2) (a product of two series in 2D); U[1e3, 1e5]
    uniform query points per table."""
    rng = np.random.default_rng(seed)
    specs, values, counts = [], [], []
    for i in range(ntables):
        order = int(rng.choice([3, 5]))
        periodic = bool(rng.random() < 0.3)
        if i % 2 == 0:
            dims = [int(rng.integers(16, 4097))]
            v = _fourier(rng, dims[0], periodic)
        else:
            dims = [int(rng.integers(16, 257)), int(rng.integers(16, 257))]
            v = np.outer(_fourier(rng, dims[0], periodic), _fourier(rng, dims[1], periodic))
        specs.append((order, [periodic] * len(dims), dims, [(0.0, float(d)) for d in dims]))
        values.append(v.ravel())
        counts.append(int(rng.integers(1000, 100001)))
    return specs, np.concatenate(values), np.asarray(counts, np.int64)


def run_batched(args, torch, steps=5, warmup=3):
    """Batched-tables workload: one build of every table and one evaluation
    of every table's points per step (FP32 evaluation, double-word solve),
    inputs resident in HBM; CUDA-event timing."""
    import bsplineinterpolation_gb300 as bi
    specs, values, counts = make_batched_workload(args.batched_tables, SEED + 2)
    b = bi.TableBatch(specs, precision="mixed")
    vals = torch.tensor(values, device="cuda")
    offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(SEED + 3)
    dims = [len(sp[2]) for sp in specs]
    parts = []
    for i, sp in enumerate(specs):
        scale = torch.tensor([float(d) for d in sp[2]], device="cuda", dtype=torch.float64)
        parts.append((torch.rand((int(counts[i]), dims[i]), device="cuda", dtype=torch.float64,
                                 generator=gen) * scale).reshape(-1))
    coords = torch.cat(parts)
    del parts
    npts = int(offsets[-1])
    out = torch.empty((npts, 1), device="cuda", dtype=torch.float32)
    # the line solves' schedule for this batch (work queue, staging budget,
    # lines per item), chosen by timing each candidate build once
    schedule = b.autotune(vals)
    for _ in range(warmup):
        b.build(vals)
        b.evaluate(coords, offsets, out=out)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for e0, e1, e2 in ev:
        e0.record()
        b.build(vals)
        e1.record()
        b.evaluate(coords, offsets, out=out)
        e2.record()
    torch.cuda.synchronize()
    build_ms = float(np.median([a.elapsed_time(c) for a, c, _ in ev]))
    eval_ms = float(np.median([c.elapsed_time(d) for _, c, d in ev]))
    total_ms = ev[0][0].elapsed_time(ev[-1][2]) / steps
    # the same step replayed from a captured CUDA graph (intp_batch_graph_*)
    g = b.graph(vals, coords, offsets, out=out)
    for _ in range(warmup):
        g.launch(torch.cuda.current_stream())
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record()
    for _ in range(steps):
        g.launch(torch.cuda.current_stream())
    g1.record()
    torch.cuda.synchronize()
    graph_ms = g0.elapsed_time(g1) / steps
    g.close()
    # accuracy of a sample of tables against the FP64 form of the same batch
    b64 = bi.TableBatch(specs, precision="fp64")
    b64.build(vals)
    ref = b64.evaluate(coords, offsets, out_dtype="f64")
    err = float(((out[:, 0].double() - ref[:, 0]).abs().max() / ref[:, 0].abs().max()).item())
    return {"workload": "%d tables (half 1D N~U[16,4096], half 2D sides~U[16,256]; O in {3,5}; 30%% periodic),"
                        " %d queries" % (len(specs), npts),
            "points_per_s": npts / (total_ms / 1e3), "build_ms": build_ms, "eval_ms": eval_ms,
            "graph_ms": graph_ms, "graph_points_per_s": npts / (graph_ms / 1e3),
            "eval_points_per_s": npts / (eval_ms / 1e3), "mesh_values": int(values.size),
            "max_rel_err_vs_fp64": err, "steps": steps, "warmup": warmup, "schedule": schedule}


# ---------------------------------------------------------------------------
# serving loop: Poisson arrivals of builds and evaluations
# ---------------------------------------------------------------------------
def run_serving(args, torch, rate=2000.0, seed=SEED + 4):
    """Serving-loop workload: Poisson arrivals at `rate` requests/s for
    --serve-seconds; 10% table builds (2D 32^2..1024^2 or 3D 64^3..256^3,
    order 3 or 5, random periodicity, values exp(-r^2) cos(4x) + noise on
    [-1, 1]^D), 90% evaluations of 1e3..1e7 log-uniform uniform points against
    built tables; 150 GB memory budget with LRU eviction. Latency is measured
    by the server from submission to completion on the device. Inputs come
    from page-locked host pools (intp_host_alloc; a build's values and an
    evaluation's points are slices of them)."""
    import bsplineinterpolation_gb300 as bi
    rng = np.random.default_rng(seed)
    # pools: value meshes of a few sizes per class, points, outputs
    def pinned(a):
        # page-locked host memory from the library's host allocator
        h = bi.host_empty(a.shape, a.dtype)
        h[...] = a
        return torch.from_numpy(h)

    def mesh(dims):
        axes = np.meshgrid(*[np.linspace(-1.0, 1.0, d) for d in dims], indexing="ij")
        r2 = sum(a * a for a in axes)
        f = np.exp(-r2) * np.cos(4 * axes[0]) + rng.normal(0.0, 1e-3, dims)
        return pinned(f)
    pool2 = [mesh([int(v), int(v)]) for v in (32, 128, 256, 512, 768, 1024)]
    pool3 = [mesh([int(v)] * 3) for v in (64, 96, 128, 192, 256)]
    max_pts = 10_000_000
    pts3 = pinned(rng.uniform(-1.0, 1.0, (max_pts, 3)))
    pts2 = pinned(np.ascontiguousarray(pts3.numpy()[:, :2]))
    ring = torch.from_numpy(bi.host_empty((1 << 28,), np.float32))  # output ring
    trace_seed = seed + 1

    def one_run():
        """One run of the seeded arrival trace against a fresh server."""
        rng = np.random.default_rng(trace_seed)
        srv = bi.Server(memory_budget=150 << 30, slots=args.serve_slots)
        tables = []  # (table id, dim)
        ring_pos = [0]

        def submit_build():
            if rng.random() < 0.5:
                v = pool2[int(rng.integers(len(pool2)))]
            else:
                v = pool3[int(rng.integers(len(pool3)))]
            D = v.dim()
            per = [bool(rng.random() < 0.5) for _ in range(D)]
            tid, rid = srv.submit_build(int(rng.choice([3, 5])), per, v, *[(-1.0, 1.0)] * D)
            tables.append((tid, D))
            return rid

        def submit_eval():
            tid, D = tables[int(rng.integers(max(0, len(tables) - 64), len(tables)))]
            n = int(np.exp(rng.uniform(np.log(1e3), np.log(1e7))))
            o = int(rng.integers(0, max_pts - n + 1))
            p = (pts3 if D == 3 else pts2)[o:o + n]
            if ring_pos[0] + n > ring.numel():
                ring_pos[0] = 0
            out = ring[ring_pos[0]:ring_pos[0] + n].view(n, 1)
            ring_pos[0] += n
            return srv.submit_eval(tid, p, out)

        rids = [submit_build() for _ in range(16)]
        for r in rids:
            srv.wait(r, 300.0)
        srv.reset_stats()
        rids = []
        t0 = time.perf_counter()
        t_next = t0
        while True:
            t_next += rng.exponential(1.0 / rate)
            if t_next - t0 > args.serve_seconds:
                break
            now = time.perf_counter()
            if t_next > now:
                time.sleep(t_next - now)
            rids.append(submit_build() if rng.random() < 0.1 else submit_eval())
        statuses = [srv.wait(r, 600.0) for r in rids]
        wall = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        return rids, statuses, wall, st

    runs = [one_run() for _ in range(max(1, args.serve_runs))]
    rids, statuses, wall, st = runs[0]
    p99s = [r[3]["all_p99_ms"] for r in runs]
    return {"workload": "Poisson %.0f req/s for %.0f s: 10%% builds (2D 32^2-1024^2 / 3D 64^3-256^3, O 3|5),"
                        " 90%% evals of 1e3-1e7 points; 150 GB budget, %d slots" % (rate, args.serve_seconds,
                                                                                     args.serve_slots),
            "requests": len(rids), "failed": int(sum(1 for r in runs for x in r[1] if x != 0)),
            "p50_ms": st["all_p50_ms"], "p99_ms": st["all_p99_ms"],
            "p99_ms_runs": p99s, "p99_ms_max": max(p99s), "runs": len(runs),
            "eval_p50_ms": st["eval_p50_ms"], "eval_p99_ms": st["eval_p99_ms"],
            "build_p50_ms": st["build_p50_ms"], "build_p99_ms": st["build_p99_ms"],
            "points_per_s": st["points_per_s"], "points": st["points_evaluated"],
            "merged_units": st["merged_units"], "evictions": st["evictions"],
            "served_points_per_wall_s": st["points_evaluated"] / max(wall, 1e-9)}


def run_reference(args, rank, world):
    """The reference arm: the reference's own CPU code (headers compiled with
    g++ -O3 INTP_MULTITHREAD; the faster of its two control-point layouts) on
    whole steps of the 3D cubic workload, all host threads. A step is the
    reference constructor at 256^3 (knots, factors, solve on its thread pool)
    plus value and d/dx at every one of the 1e8 points (operator() and
    derivative(), the points split over the host threads). Warm-up steps run
    on a 1e6-point sample. Timed steps stop once --ref-seconds have passed
    (at least one); `steps` reports how many were timed."""
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(SEED)
    n, npts = args.mesh, args.npts
    vals = make_values_np(n, rng)
    pts = make_points_np(npts, rng)
    lo, hi = [-1.0] * 3, [1.0] * 3
    out = np.empty((npts, len(DERIVS)), np.float64)
    if _reference_available():
        from oracle import reference
        layout, _ = _pick_layout(3, [False] * 3, vals, lo, hi, pts[:1_000_000], DERIVS, threads, npts)
        kind, what = "reference", "reference headers (g++ -O3 INTP_MULTITHREAD, %s layout)" % layout

        def step(m):
            t0 = time.perf_counter()
            f = reference.RefFunction(3, [False] * 3, vals, lo, hi, layout=layout)
            f.outputs(pts[:m], DERIVS, nthreads=threads, out=out[:m])
            return time.perf_counter() - t0
    else:
        from oracle import oracle
        kind, what = "port", "C restatement of the reference (reference build unavailable)"

        def step(m):
            t0 = time.perf_counter()
            s = oracle.Spline(3, 3, [0, 0, 0], [n] * 3, lo, hi)
            s.interpolate(vals, nthreads=threads)
            out[:m] = s.derivative(pts[:m], DERIVS, nthreads=threads)
            return time.perf_counter() - t0
    for _ in range(max(0, args.warmup)):
        step(min(npts, 1_000_000))
    times = []
    t_start = time.perf_counter()
    while len(times) < max(1, args.steps):
        times.append(step(npts))
        if time.perf_counter() - t_start > args.ref_seconds:
            break
    steps = len(times)
    total = sum(times)
    res = {
        "metric": METRIC, "value": npts * steps / total, "unit": "points/s", "n_gpus": world,
        "steps": steps, "warmup": args.warmup, "ms_per_step": total / steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded; shapes and distributions of the 3D cubic workload)",
        "config": {"workload": "3D cubic 256^3 build + 1e8 queries value+d/dx", "mesh": [n] * 3,
                   "order": 3, "queries": npts, "precision": "fp64", "parallelism": "host threads",
                   "steps_requested": args.steps},
        "impl": "reference",
    }
    res["cpu_baseline"] = {"value": res["value"], "unit": "points/s", "cores": threads, "kind": kind,
                           "sample": "%s: %d whole steps (build + all %d points), warm-up steps on 1e6 points"
                                     % (what, steps, npts)}
    res["e2e"] = {"value": res["value"], "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    if not args.no_configs:
        for cfg in (CFG1, CFG4):
            v, p = config_inputs(cfg)
            timing, _ = config_cpu(cfg, v, p)
            res[cfg["name"]] = dict(workload=cfg["workload"], points=int(p.shape[0]), **timing)
    return res


def main():
    args = parse()
    if args.batched_only or args.serve_only:
        import torch
        res = run_batched(args, torch) if args.batched_only else run_serving(args, torch)
        print(json.dumps(res), flush=True)
        return
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", args.gpus if args.gpus else 1))
    if args.impl == "reference":
        res = run_reference(args, rank, world)
    else:
        res = run_ours(args, rank, world)
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
