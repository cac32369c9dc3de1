#!/usr/bin/env python
"""Kernel pair-evaluations per second of GSKS on GB300.

Workload (the general-stride configuration of the benchmark spec): a pool of
N = 262144 points in k = 64 dimensions drawn uniform[0,1] (FP64), m = n =
65536 targets / sources chosen as random subsets of the pool (amap, bmap),
u / w maps random permutations of [0, 65536), weights N(0,1).  One step
evaluates the three kernels of that configuration on it, each a full
m x n summation into u:
    Gaussian h = 0.5 (scal = -1/(2h^2) = -2), Laplace (powe, scal from k),
    polynomial (scal = 1/k, cons = 1, powe = 3).
Synthetic, seeded inputs of the specified shapes and distributions.

Reported:
  value     pair-evals/s over the timed steps, inputs resident in HBM, through
            gsks_dgsks_device (CUDA events on the launch stream, L2 flushed
            between steps by a 512 MiB memset);
  e2e       the same through ks.h dgsks() with host arrays: gather, host->device
            copies, kernels and the device->host copy of u inside the region;
  roofline  per kernel type against the measured pipe rate that binds it;
  cpu_baseline  the CPU port of the reference's fused dgsks (oracle) on all
            host cores, on sampled target rows x all sources; its row sums
            also give the error of the GPU result on those rows.
  --impl reference times that CPU implementation alone (the reference's own
  code does not build on the aarch64 host: its micro-kernels are AVX).

Multi-GPU (torchrun): every rank runs an independent replica of the workload
(no data-path collective); value = all pairs / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "kernel pair-evals/s, split-TC vs FP64 GPU at <=1e-6 rel err; % of roofline"
N_POOL, K_DIM, M_T, N_S = 262144, 64, 65536, 65536
# reference per-pair flop model (test/test_dgsks.c:254-283): 2k + f_type
KERNELS = [
    ("gaussian", 0, dict(scal=-2.0), 37),
    ("laplace", 2, {}, 60),
    ("polynomial", 1, dict(scal=1.0 / K_DIM, cons=1.0, powe=3.0), 6),
]
WORKLOAD = ("general stride: pool 262144 x k=64 uniform[0,1] FP64; m=n=65536 random subsets; "
            "u/w maps random permutations of [0,65536); Gaussian h=0.5 + Laplace + polynomial pwr=3")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "split"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--case", default=None, choices=[k[0] for k in KERNELS],
                    help="profiling case: only device calls of one kernel type (for ncu)")
    ap.add_argument("--m", type=int, default=M_T)
    ap.add_argument("--n", type=int, default=N_S)
    ap.add_argument("--reps", type=int, default=2)
    return ap.parse_args()


def run_case(args):
    """A small device-resident case of one kernel type, for ncu captures: the
    configuration's pool and k, m x n targets/sources, `reps` calls."""
    import torch
    from ks_gb300 import build as B
    if not os.path.exists(B.LIB):
        B.build()
    from ks_gb300 import gsks
    torch.cuda.set_device(0)
    wl = make_workload(torch)
    prec = gsks.GSKS_FP64 if args.precision == "fp64" else gsks.GSKS_SPLIT_BF16X3
    name, kt, p, _f = [k for k in KERNELS if k[0] == args.case][0]
    u = torch.zeros(M_T, dtype=torch.float64, device="cuda")
    for _ in range(args.reps):
        gsks.dgsks_device(gsks.make_kernel(kt, **p), args.m, args.n, K_DIM, u, wl["umap"], wl["X"], wl["X2"],
                          wl["amap"], wl["X"], wl["X2"], wl["bmap"], wl["w"], wl["wmap"], precision=prec,
                          stream=torch.cuda.current_stream(), nxa=N_POOL, nxb=N_POOL)
    torch.cuda.synchronize()
    print(json.dumps({"case": name, "m": args.m, "n": args.n, "reps": args.reps, "precision": args.precision,
                      "u_norm": float(u.norm())}))


# ---------------------------------------------------------------------------
def dist_setup(args):
    import torch
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, x: float) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1])); mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
def make_workload(torch, seed=1234):
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    dev = "cuda"
    X = torch.rand(N_POOL, K_DIM, dtype=torch.float64, device=dev, generator=g)
    X2 = torch.empty(N_POOL, dtype=torch.float64, device=dev)
    from ks_gb300 import gsks
    gsks.norms_device(X, X2, stream=torch.cuda.current_stream())
    amap = torch.randperm(N_POOL, device=dev, generator=g)[:M_T].to(torch.int32)
    bmap = torch.randperm(N_POOL, device=dev, generator=g)[:N_S].to(torch.int32)
    umap = torch.randperm(M_T, device=dev, generator=g).to(torch.int32)
    wmap = torch.randperm(N_S, device=dev, generator=g).to(torch.int32)
    w = torch.randn(N_S, dtype=torch.float64, device=dev, generator=g)
    torch.cuda.synchronize()
    return dict(X=X, X2=X2, amap=amap, bmap=bmap, umap=umap, wmap=wmap, w=w)


def kernel_desc(gsks, ktype, params):
    return gsks.make_kernel(ktype, **params)


def run_ours(args, ws, rank, local):
    import numpy as np
    import torch
    from ks_gb300 import build as B
    if not os.path.exists(B.LIB):
        B.build()
    from ks_gb300 import gsks
    lib = gsks.load()
    prec = gsks.GSKS_FP64 if args.precision == "fp64" else gsks.GSKS_SPLIT_BF16X3
    wl = make_workload(torch)
    stream = torch.cuda.current_stream()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    # measured pipe rates for the roofline
    dfma = C.c_double()
    lib.gsks_probe_peak(0, C.byref(dfma))
    fp64_peak = 2.0 * dfma.value  # flop/s

    def one_call(ktype, params, u):
        gsks.dgsks_device(kernel_desc(gsks, ktype, params), M_T, N_S, K_DIM, u, wl["umap"], wl["X"], wl["X2"],
                          wl["amap"], wl["X"], wl["X2"], wl["bmap"], wl["w"], wl["wmap"], precision=prec,
                          stream=stream, nxa=N_POOL, nxb=N_POOL)
        return gsks.last_launch_count()

    u = torch.zeros(M_T, dtype=torch.float64, device="cuda")
    for _ in range(args.warmup):
        for _, kt, p, _f in KERNELS:
            one_call(kt, p, u)
    torch.cuda.synchronize()

    evs = {name: [] for name, *_ in KERNELS}
    launches = 0
    barrier(ws)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for s in range(args.steps):
            flush.zero_()
            for name, kt, p, _f in KERNELS:
                a = torch.cuda.Event(enable_timing=True); b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                launches += one_call(kt, p, u)
                b.record(stream)
                evs[name].append((a, b))
            launches += 1  # the L2 flush memset
        t1.record(stream)
        torch.cuda.synchronize()
    barrier(ws)
    ms_local = t0.elapsed_time(t1)
    ms = max_over_ranks(ws, ms_local)
    pairs_step = len(KERNELS) * M_T * N_S
    value = pairs_step * args.steps * ws / (ms * 1e-3)

    # roofline per kernel type
    per = {}
    for name, kt, p, f in KERNELS:
        dur = statistics.mean(a.elapsed_time(b) for a, b in evs[name]) * 1e-3
        flops = M_T * N_S * (2 * K_DIM + f)
        per[name] = {"ms": dur * 1e3, "pairs_per_s": M_T * N_S / dur, "flops_alg": flops,
                     "achieved_tflops": flops / dur / 1e12, "frac": flops / dur / fp64_peak}
    dominant = max(per, key=lambda k: per[k]["ms"])
    traffic = read_traffic(dominant)
    roof = {"bound": "fp64", "kernel": f"fp64_tiles<{dominant}> + fp64_reduce",
            "achieved": round(per[dominant]["achieved_tflops"], 4), "peak": round(fp64_peak / 1e12, 4),
            "unit": "TFLOP/s", "frac": round(per[dominant]["frac"], 4), "traffic": traffic,
            "peak_source": "measured live: gsks_probe_peak FP64 FMA issue rate x 2 (no FP64 entry in MEASURED_PEAKS.json)",
            "flop_model": "m*n*(2k + f_type), f_type from test/test_dgsks.c:254-283",
            "per_kernel": {k: {kk: (round(vv, 5) if isinstance(vv, float) else vv) for kk, vv in v.items()}
                           for k, v in per.items()}}

    line = {
        "metric": METRIC, "value": value, "unit": "pair-evals/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "bf16x3+f32+f64",
        "data": "synthetic: seeded uniform[0,1]^64 pool, N(0,1) weights, random subset / permutation maps",
        "config": {"workload": WORKLOAD, "precision": args.precision, "pool": N_POOL, "k": K_DIM,
                   "m": M_T, "n": N_S, "kernels": [k[0] for k in KERNELS],
                   "l2": "flushed between steps (512 MiB memset inside the timed region)",
                   "parallelism": f"replicas x{ws}"},
        "roofline": roof,
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }

    # error of the GPU result on sampled rows + CPU baseline (rank 0, N=1 only)
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu, err = cpu_baseline_and_error(args, torch, gsks, wl, prec, stream)
        line["cpu_baseline"] = cpu
        line["error"] = err
    if not args.no_e2e:
        line["e2e"] = run_e2e(args, torch, gsks, wl, ws)
    return line


def read_traffic(kernel_name):
    """DRAM bytes per launch from the committed ncu summary, if one exists."""
    path = os.path.join(ROOT, "profiles", f"fp64_tiles_{kernel_name}_c2.md")
    if not os.path.exists(path):
        return None
    for l in open(path):
        if l.startswith("traffic_bytes_per_launch:"):
            try:
                return float(l.split(":", 1)[1])
            except ValueError:
                return None
    return None


def run_e2e(args, torch, gsks, wl, ws):
    """Same steps through ks.h dgsks() with host (numpy) arrays."""
    import numpy as np
    h = {k: v.cpu().numpy() for k, v in wl.items()}
    u = np.zeros(M_T)
    steps = max(1, args.steps)
    for _ in range(1):
        for _, kt, p, _f in KERNELS:
            rc = gsks.dgsks_status(kernel_desc(gsks, kt, p), u, h["umap"], h["X"], h["X2"], h["amap"], h["X"],
                                   h["X2"], h["bmap"], h["w"], h["wmap"])
            assert rc == 0, gsks.error_string(rc)
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(steps):
        for _, kt, p, _f in KERNELS:
            gsks.dgsks_status(kernel_desc(gsks, kt, p), u, h["umap"], h["X"], h["X2"], h["amap"], h["X"],
                              h["X2"], h["bmap"], h["w"], h["wmap"])
    dt = max_over_ranks(ws, time.perf_counter() - t0)
    # bytes the host path copies per call: gathered A and B rows, norms, w, u in; u out
    h2d_call = 8 * (M_T * K_DIM + N_S * K_DIM + M_T + N_S + N_S + M_T)
    h2d_poly = 8 * (M_T * K_DIM + N_S * K_DIM + N_S + M_T)  # no norms for the inner-product kernel
    h2d = 2 * h2d_call + h2d_poly
    return {"value": len(KERNELS) * M_T * N_S * steps * ws / dt, "unit": "pair-evals/s",
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 8 * M_T * len(KERNELS),
            "path": "ks.h dgsks() with host numpy arrays (pinned staging inside the call)"}


def cpu_baseline_and_error(args, torch, gsks, wl, prec, stream):
    """CPU port of the reference's fused dgsks on sampled rows x all sources, all
    host cores; the same row sums measure the GPU result's error."""
    import numpy as np
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    h = {k: v.cpu().numpy() for k, v in wl.items()}
    # The checker's norms are summed in the order of its own inner products, so
    # that coincident pool points cancel exactly there (Laplace is singular at
    # d2 = 0, frame/dgsks_ref.c:343-345); the GPU used its device-computed norms.
    h["X2"] = O.norms(h["X"])
    # one fresh GPU evaluation of each kernel into its own u for the comparison
    gpu_u = {}
    for name, kt, p, _f in KERNELS:
        u = torch.zeros(M_T, dtype=torch.float64, device="cuda")
        gsks.dgsks_device(kernel_desc(gsks, kt, p), M_T, N_S, K_DIM, u, wl["umap"], wl["X"], wl["X2"], wl["amap"],
                          wl["X"], wl["X2"], wl["bmap"], wl["w"], wl["wmap"], precision=prec, stream=stream)
        torch.cuda.synchronize()
        gpu_u[name] = u.cpu().numpy()
    # calibrate the sample to about args.cpu_seconds of CPU work
    rng = np.random.default_rng(7)
    def timed(rows):
        t = 0.0
        outs = {}
        for name, kt, p, _f in KERNELS:
            amap_s = np.ascontiguousarray(h["amap"][rows])
            umap_s = np.arange(rows.size, dtype=np.int32)
            u_s = np.zeros(rows.size)
            t0 = time.perf_counter()
            O.dgsks(O.make_kernel(kt, **p), u_s, umap_s, h["X"], h["X2"], amap_s, h["X"], h["X2"], h["bmap"],
                    h["w"], h["wmap"], impl="fused")
            t += time.perf_counter() - t0
            outs[name] = u_s
        return t, outs
    rows0 = np.sort(rng.choice(M_T, 64, replace=False)).astype(np.int32)
    t0, _ = timed(rows0)
    S = int(min(M_T, max(64, 64 * args.cpu_seconds / max(t0, 1e-3))))
    rows = np.sort(rng.choice(M_T, S, replace=False)).astype(np.int32)
    t, outs = timed(rows)
    pairs = len(KERNELS) * S * N_S
    cpu = {"value": pairs / t, "unit": "pair-evals/s", "cores": cores, "kind": "port",
           "sample": f"{S} random target rows x all {N_S} sources, each of the {len(KERNELS)} kernels "
                     f"({pairs:.3g} pairs, {t:.1f} s)",
           "impl": "oracle_dgsks_fused (C restatement of frame/dgsks.c, OpenMP); the reference's AVX "
                   "micro-kernels do not build on aarch64"}
    err = {}
    for name, kt, p, _f in KERNELS:
        _, cond = O.rows(O.make_kernel(kt, **p), rows, h["X"], h["X2"], h["amap"], h["X"], h["X2"], h["bmap"],
                         h["w"], h["wmap"])
        ug = gpu_u[name][h["umap"][rows]]
        e = O.errors(ug, outs[name], cond=cond)
        err[name] = {k: float("%.3g" % v) for k, v in e.items()}
    err["rows_checked"] = int(S)
    return cpu, err


def run_reference(args, ws, rank):
    """The reference's CPU implementation of the path on this host's cores: the
    oracle port of its fused dgsks (the reference's AVX micro-kernels do not
    build on aarch64), bounded sample per step."""
    import numpy as np
    if rank != 0:
        return None
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    rng = np.random.default_rng(1234)
    X = rng.random((N_POOL, K_DIM))
    X2 = O.norms(X)
    amap = rng.permutation(N_POOL)[:M_T].astype(np.int32)
    bmap = rng.permutation(N_POOL)[:N_S].astype(np.int32)
    wmap = rng.permutation(N_S).astype(np.int32)
    w = rng.standard_normal(N_S)

    def step(S):
        rows = np.sort(rng.choice(M_T, S, replace=False)).astype(np.int32)
        for _, kt, p, _f in KERNELS:
            u = np.zeros(S)
            O.dgsks(O.make_kernel(kt, **p), u, np.arange(S, dtype=np.int32), X, X2,
                    np.ascontiguousarray(amap[rows]), X, X2, bmap, w, wmap, impl="fused")
    t0 = time.perf_counter(); step(32); t1 = time.perf_counter() - t0
    budget = 120.0 / max(1, args.steps + args.warmup)   # whole run within a few minutes
    S = int(min(M_T, max(32, 32 * min(budget, 15.0) / max(t1, 1e-3))))
    for _ in range(args.warmup):
        step(S)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step(S)
    dt = time.perf_counter() - t0
    pairs = len(KERNELS) * S * N_S * args.steps
    v = pairs / dt
    return {"metric": METRIC, "value": v, "unit": "pair-evals/s", "impl": "reference", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: seeded uniform[0,1]^64 pool, N(0,1) weights",
            "config": {"workload": WORKLOAD, "precision": "fp64", "sample_rows_per_step": S},
            "cpu_baseline": {"value": v, "unit": "pair-evals/s", "cores": cores, "kind": "port",
                             "sample": f"{S} random target rows x all {N_S} sources x {len(KERNELS)} kernels per step"},
            "e2e": {"value": v, "unit": "pair-evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    if args.case:
        run_case(args)
        return
    if args.impl == "reference":
        ws = int(os.environ.get("WORLD_SIZE", "1")); rank = int(os.environ.get("RANK", "0"))
        line = run_reference(args, ws, rank)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    ws, rank, local = dist_setup(args)
    line = run_ours(args, ws, rank, local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
