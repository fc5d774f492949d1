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
`--impl reference` times the reference algorithm on the host cores (the C
restatement of the reference, multithreaded) on a bounded sample.
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
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64-form comparison")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer measurement")
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
# CPU baseline (reference algorithm on the host cores)
# ---------------------------------------------------------------------------
def cpu_baseline(npts_step, mesh_n, sample_pts, gpu_check=None):
    """Times the reference algorithm (C restatement, all host threads) on a
    bounded sample: the full mesh solve plus `sample_pts` evaluations of
    value and d/dx; the step time is extrapolated to npts_step points."""
    from oracle import oracle
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(SEED)
    vals = make_values_np(mesh_n, rng)
    pts = make_points_np(sample_pts, rng)
    s = oracle.Spline(3, 3, [0, 0, 0], [mesh_n] * 3, [-1.0] * 3, [1.0] * 3)
    t0 = time.perf_counter()
    s.interpolate(vals, nthreads=threads)
    t1 = time.perf_counter()
    out = s.derivative(pts, DERIVS, nthreads=threads)
    t2 = time.perf_counter()
    solve_s = t1 - t0
    eval_s = (t2 - t1) * npts_step / sample_pts
    res = {
        "value": npts_step / (solve_s + eval_s),
        "unit": "points/s",
        "cores": threads,
        "kind": "port",
        "sample": "full %d^3 solve + %d of %d points (value and d/dx), step time extrapolated"
                  % (mesh_n, sample_pts, npts_step),
        "solve_ms": solve_s * 1e3,
        "eval_points_per_s": sample_pts / (t2 - t1),
    }
    if gpu_check is not None:
        res["_check"] = (vals, pts, out)
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
                                        precision=precision)

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
                   "outputs": ["value", "d/dx"], "precision": prec,
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
        result["fp64_plain"] = {"points_per_s": npts * 2 / (tot64 / 1e3),
                                "solve_ms": float(np.median(s64)), "eval_ms": float(np.median(e64))}
        result["mixed_max_rel_err_vs_fp64"] = {"value": errs[0], "d/dx": errs[1],
                                               "norm": "max|err| / max|fp64| over all queries"}
        del f64, out64

    if rank == 0 and not args.no_e2e:
        result["e2e"] = e2e(args, f, vals, pts, lib, torch)
    if rank == 0 and not args.no_cpu:
        result["cpu_baseline"] = cpu_baseline(npts, n, min(npts, 20_000_000))
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return result


def e2e(args, f, vals, pts, lib, torch):
    """Same metric through the C-ABI with host buffers: the step copies the
    values and coordinates from pinned host memory, solves, evaluates and
    copies the results back."""
    npts = pts.shape[0]
    K = len(DERIVS)
    hv = vals.cpu().pin_memory()
    hp = pts.cpu().pin_memory()
    od = _out_dtype(args)
    ho = torch.empty((npts, K), dtype=torch.float32 if od == 1 else torch.float64).pin_memory()
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
    steps = max(1, min(args.steps, 3))
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


def run_reference(args, rank, world):
    if rank != 0:
        return None
    base = cpu_baseline(args.npts, args.mesh, min(args.npts, 10_000_000))
    steps = max(1, args.steps)
    return {
        "metric": METRIC, "value": base["value"], "unit": "points/s", "n_gpus": world,
        "steps": steps, "warmup": args.warmup,
        "ms_per_step": args.npts / base["value"] * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded; shapes and distributions of the 3D cubic workload)",
        "config": {"workload": "3D cubic 256^3 build + 1e8 queries value+d/dx", "mesh": [args.mesh] * 3,
                   "order": 3, "queries": args.npts, "precision": "fp64",
                   "parallelism": "host threads"},
        "impl": "reference",
        "cpu_baseline": {k: base[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": base["value"], "unit": "points/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main():
    args = parse()
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
