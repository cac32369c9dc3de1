#!/usr/bin/env python
"""Kernel pair-evaluations per second of GSKS on GB300: split-precision
tensor-core form against the plain FP64 form, with errors and rooflines.

Workload (the general-stride configuration of the benchmark spec): a pool of
N = 262144 points in k = 64 dimensions drawn uniform[0,1] (FP64), m = n =
65536 targets / sources chosen as random subsets of the pool (amap, bmap),
u / w maps random permutations of [0, 65536), weights N(0,1).  One step
evaluates the three kernels of that configuration, each a full m x n
summation into u: Gaussian h = 0.5 (scal = -1/(2h^2) = -2), Laplace (powe,
scal from k), polynomial (scal = 1/k, cons = 1, powe = 3).  Synthetic, seeded
inputs of the specified shapes and distributions.

Reported (one JSON line):
  value      pair-evals/s of the split-precision form, inputs resident in HBM,
             through gsks_dgsks_device (CUDA events on the launch stream, L2
             flushed between steps by a 512 MiB memset inside the region);
  forms      the same for the split and the plain FP64 form, their ratio and
             their per-kernel times;
  e2e        the split form through ks.h dgsks() with host arrays (gather,
             host->device copies, kernels, device->host copy of u);
  roofline   per form and kernel against the measured pipe that binds it;
  cpu_baseline  the oracle's port of the reference's fused dgsks on all host
             cores over sampled target rows x all sources; its row sums also
             give the errors of both forms (normwise and conditioned).
  list       the batched configuration (20000 tasks over a 1M-point pool,
             k = 16, mixed kernels) through dgsks_list in both forms, with
             errors on a task subset and the oracle's OpenMP list driver as
             CPU baseline (skipped with --no-list).
  --impl reference times that CPU implementation alone (the reference's own
  micro-kernels are AVX and do not build on the aarch64 host).

Multi-GPU (torchrun): every rank runs an independent replica (no data-path
collective); value = all ranks' pairs / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
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
SPLIT_PRODUCTS = 6   # tensor-core products per slice pair set (a1b1, a1b2, a2b1, a2b2, a1b3, a3b1)

# The batched configuration (dgsks_list), reported beside the headline.
LIST_POOL, LIST_K, LIST_TASKS = 1 << 20, 16, 20000
LIST_WORKLOAD = ("batched dgsks_list: 20000 independent (amap, bmap) pairs over a pool of 1,048,576 points in "
                 "k=16 uniform[0,1]; list sizes log-uniform in [32, 4096]; kernel per task drawn from {Gaussian "
                 "h~U[0.1,2], Laplace, polynomial pwr 2 or 3 (scal 1/k, cons 1)}; w ~ N(0,1)")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--forms", default="split,fp64", help="forms to time; the first is the headline")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--case", default=None, choices=[k[0] for k in KERNELS] + ["list"],
                    help="profiling case: only device calls of one kernel type, or the batched "
                         "workload with --tasks tasks (for ncu)")
    ap.add_argument("--tasks", type=int, default=2000, help="tasks of --case list")
    ap.add_argument("--precision", default="split", choices=["fp64", "split"], help="form of --case")
    ap.add_argument("--m", type=int, default=M_T)
    ap.add_argument("--n", type=int, default=N_S)
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--no-list", action="store_true", help="skip the batched (dgsks_list) section")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the other configurations (mixture k=3/512, variable bandwidth, dense k=1024)")
    ap.add_argument("--config", default=None, choices=["c3", "c5a", "c5b"],
                    help="one of the other benchmark configurations instead of the default line: c3 (mixture, "
                         "k swept), c5a (variable bandwidth, 2^20 points), c5b (k = 1024 polynomial)")
    return ap.parse_args()


def peaks_file():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


# ---------------------------------------------------------------------------
def dist_setup():
    import torch
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="nccl" if torch.cuda.is_available() else "gloo")
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


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.proc, self.lines = index, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines += [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
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
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
def make_workload(torch, seed=1234):
    from ks_gb300 import gsks
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    X = torch.rand(N_POOL, K_DIM, dtype=torch.float64, device="cuda", generator=g)
    X2 = torch.empty(N_POOL, dtype=torch.float64, device="cuda")
    gsks.norms_device(X, X2, stream=torch.cuda.current_stream())
    amap = torch.randperm(N_POOL, device="cuda", generator=g)[:M_T].to(torch.int32)
    bmap = torch.randperm(N_POOL, device="cuda", generator=g)[:N_S].to(torch.int32)
    umap = torch.randperm(M_T, device="cuda", generator=g).to(torch.int32)
    wmap = torch.randperm(N_S, device="cuda", generator=g).to(torch.int32)
    w = torch.randn(N_S, dtype=torch.float64, device="cuda", generator=g)
    torch.cuda.synchronize()
    return dict(X=X, X2=X2, amap=amap, bmap=bmap, umap=umap, wmap=wmap, w=w)


def prec_of(gsks, form):
    return gsks.GSKS_FP64 if form == "fp64" else gsks.GSKS_SPLIT_BF16X3


def device_call(gsks, wl, kt, p, u, prec, stream, m=M_T, n=N_S):
    gsks.dgsks_device(gsks.make_kernel(kt, **p), m, n, K_DIM, u, wl["umap"], wl["X"], wl["X2"], wl["amap"],
                      wl["X"], wl["X2"], wl["bmap"], wl["w"], wl["wmap"], precision=prec, stream=stream,
                      nxa=N_POOL, nxb=N_POOL)
    return gsks.last_launch_count()


def run_case(args):
    """A device-resident case of one kernel type, for ncu captures."""
    import torch
    from ks_gb300 import build as B
    if not os.path.exists(B.LIB):
        B.build()
    from ks_gb300 import gsks
    torch.cuda.set_device(0)
    if args.case == "list":
        import numpy as np
        L = make_list_workload(ntask=args.tasks)
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        X, w = dev(L["X"]), dev(L["w"])
        kers = [gsks.make_kernel(t, **p) for t, p in L["specs"]]
        gsks.set_precision(prec_of(gsks, args.precision))
        u = torch.zeros(LIST_POOL, dtype=torch.float64, device="cuda")
        for _ in range(args.reps):
            gsks.dgsks_list(kers[0], u, dev(L["a_off"]), dev(L["a_idx"]), dev(L["b_off"]), dev(L["b_idx"]),
                            X, None, X, None, w, kers=kers)
        torch.cuda.synchronize()
        print(json.dumps({"case": "list", "tasks": args.tasks, "pairs": L["pairs"], "reps": args.reps,
                          "precision": args.precision, "u_norm": float(u.norm())}))
        return
    wl = make_workload(torch)
    name, kt, p, _f = [k for k in KERNELS if k[0] == args.case][0]
    u = torch.zeros(M_T, dtype=torch.float64, device="cuda")
    for _ in range(args.reps):
        device_call(gsks, wl, kt, p, u, prec_of(gsks, args.precision), torch.cuda.current_stream(), args.m, args.n)
    torch.cuda.synchronize()
    print(json.dumps({"case": name, "m": args.m, "n": args.n, "reps": args.reps, "precision": args.precision,
                      "u_norm": float(u.norm())}))


def time_form(args, torch, gsks, wl, form, ws, flush, stream, clk):
    """W warm-up + K timed steps of one form; per-kernel event times."""
    prec = prec_of(gsks, form)
    u = torch.zeros(M_T, dtype=torch.float64, device="cuda")
    for _ in range(args.warmup):
        for _, kt, p, _f in KERNELS:
            device_call(gsks, wl, kt, p, u, prec, stream)
    torch.cuda.synchronize()
    evs = {name: [] for name, *_ in KERNELS}
    launches = 0
    barrier(ws)
    torch.cuda.synchronize()
    with clk:
        t0 = torch.cuda.Event(enable_timing=True); t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(args.steps):
            flush.zero_()
            launches += 1
            for name, kt, p, _f in KERNELS:
                a = torch.cuda.Event(enable_timing=True); b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                launches += device_call(gsks, wl, kt, p, u, prec, stream)
                b.record(stream)
                evs[name].append((a, b))
        t1.record(stream)
        torch.cuda.synchronize()
    barrier(ws)
    ms = max_over_ranks(ws, t0.elapsed_time(t1))
    per = {name: statistics.mean(a.elapsed_time(b) for a, b in v) for name, v in evs.items()}
    return ms, per, launches


def roofline_split(per, peaks, rates):
    """Split form: algorithmic 2mnk at the tensor peak (and the executed split
    products), ex2 at the measured SFU rate, per kernel."""
    out = {}
    tc_peak = peaks.get("bf16_tflops", 1900.0) * 1e12
    for name, kt, p, _f in KERNELS:
        t = per[name] * 1e-3
        pairs = M_T * N_S
        alg = 2.0 * pairs * K_DIM
        execd = SPLIT_PRODUCTS * 2.0 * pairs * ((K_DIM + 15) // 16 * 16)
        t_tc, t_exec = alg / tc_peak, execd / tc_peak
        t_sfu = pairs / rates["ex2"] if kt in (0, 3) else 0.0
        bound_t = max(t_tc, t_sfu)
        out[name] = {"ms": round(per[name], 4), "pairs_per_s": pairs / t,
                     "alg_tflops": round(alg / t / 1e12, 2), "frac_alg_tensor": round(t_tc / t, 4),
                     "executed_tflops": round(execd / t / 1e12, 2), "frac_executed_tensor": round(t_exec / t, 4),
                     "frac_sfu": round(t_sfu / t, 4) if t_sfu else None,
                     "frac_of_binding": round(bound_t / t, 4)}
    return out


# FP64 pipe: ncu reports sm__inst_executed_pipe_fp64.avg.peak_sustained = 1/16
# warp instruction per SM cycle on GB300, i.e. 2 DFMA per SM per cycle; the
# FP64 tensor-core MMA (DMMA) issues to the same pipe at 1.8 FMA per SM cycle
# (profiles/fp64_pipe_peak.md).
FP64_FMA_PER_SM_CYCLE = 2.0


def fp64_peak(sms, sm_mhz):
    """FP64 flop/s peak at the sampled SM clock: 2 flops per FMA."""
    return 2.0 * FP64_FMA_PER_SM_CYCLE * sms * sm_mhz * 1e6


def roofline_fp64(per, peak):
    """FP64 form per kernel: the reference's flop model (2k + f per pair,
    test/test_dgsks.c:254-283; it counts more flops for pow/exp than binary
    powering issues, so it can exceed 1) and the rank-k part alone (2k per
    pair, every one a DFMA: a lower bound of the pipe's load)."""
    out = {}
    for name, kt, p, f in KERNELS:
        t = per[name] * 1e-3
        flops = M_T * N_S * (2 * K_DIM + f)
        rank_k = M_T * N_S * 2 * K_DIM
        out[name] = {"ms": round(per[name], 3), "pairs_per_s": M_T * N_S / t,
                     "achieved_tflops": round(flops / t / 1e12, 4), "frac": round(flops / t / peak, 4),
                     "frac_rank_k": round(rank_k / t / peak, 4)}
    return out


def read_profile_value(name, key):
    """A `key: value` line of a committed ncu summary (profiles/<name>.md)."""
    path = os.path.join(ROOT, "profiles", name + ".md")
    if not os.path.exists(path):
        return None
    for l in open(path):
        if l.startswith(key + ":"):
            try:
                return float(l.split(":", 1)[1])
            except ValueError:
                return None
    return None


def read_traffic(name):
    """DRAM bytes per launch from a committed ncu summary."""
    return read_profile_value(name, "traffic_bytes_per_launch")


def issue_bound(name, pairs, t, sm_mhz, sms):
    """Issue-rate bound of a kernel: its thread instructions per pair (ncu,
    committed summary) x pairs over the issue capacity, one warp instruction
    per cycle per SM sub-partition (SMs x 4 x clock x 32 threads)."""
    ipp = read_profile_value(name, "thread_instructions_per_pair")
    if ipp is None or not sm_mhz:
        return None
    cap = sms * 4 * sm_mhz * 1e6 * 32
    t_issue = ipp * pairs / cap
    return {"thread_instructions_per_pair": ipp, "capacity_thread_instr_per_s": cap,
            "t_issue_ms": round(t_issue * 1e3, 4), "frac": round(t_issue / t, 4),
            "source": f"profiles/{name}.md (ncu smsp__inst_executed.sum x 32 / pairs)"}


def run_ours(args, ws, rank, local):
    import torch
    from ks_gb300 import build as B
    if not os.path.exists(B.LIB):
        B.build()
    from ks_gb300 import gsks
    lib = gsks.load()
    forms = [f for f in args.forms.split(",") if f]
    wl = make_workload(torch)
    stream = torch.cuda.current_stream()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    peaks = peaks_file()
    rates = {}
    for nm, w in (("dfma", 0), ("ffma", 1), ("ex2", 2), ("dmma", 3)):
        r = C.c_double()
        lib.gsks_probe_peak(w, C.byref(r))
        rates[nm] = r.value

    clk = ClockSampler(local)
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    results, pers = {}, {}
    for form in forms:
        ms, per, launches = time_form(args, torch, gsks, wl, form, ws, flush, stream, clk)
        pairs_step = len(KERNELS) * M_T * N_S
        pers[form] = per
        results[form] = {"value": pairs_step * args.steps * ws / (ms * 1e-3), "ms_per_step": ms / args.steps,
                         "gpu_launches": launches}
    sm_mhz = clk.summary().get("sm_mhz") or 2070.0
    p64 = fp64_peak(sms, sm_mhz)
    for form in forms:
        results[form]["per_kernel"] = (roofline_split(pers[form], peaks, rates) if form == "split"
                                       else roofline_fp64(pers[form], p64))
    head = forms[0]
    H = results[head]

    # top-level roofline: the headline form's dominant kernel
    dom = max(H["per_kernel"], key=lambda k: H["per_kernel"][k]["ms"])
    dk = H["per_kernel"][dom]
    if head == "split":
        t = dk["ms"] * 1e-3
        roof = {"bound": "tensor", "kernel": f"split_tiles<{dom}>", "achieved": dk["alg_tflops"],
                "peak": round(peaks.get("bf16_tflops", 1900.0), 1), "unit": "TFLOP/s",
                "frac": dk["frac_alg_tensor"], "traffic": read_traffic(f"split_tiles_{dom}_general_stride"),
                "flops": "algorithmic 2mnk per launch; the split form executes 6 f16 products per slice set "
                         "(executed_tflops)",
                "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst; f16 runs at the bf16 rate)"
                if "bf16_tflops" in peaks else "fallback 1.9 PFLOP/s bf16"}
    else:
        roof = {"bound": "fp64", "kernel": f"fp64_tiles<{dom}>", "achieved": dk["achieved_tflops"],
                "peak": round(p64 / 1e12, 4), "unit": "TFLOP/s", "frac": dk["frac"],
                "traffic": read_traffic(f"fp64_tiles_{dom}_general_stride"),
                "peak_source": "FP64 pipe issue rate (ncu peak_sustained: 2 DFMA per SM cycle) x SMs x the "
                               "median SM clock sampled in the timed region"}
    roof["fp64_peak_tflops"] = round(p64 / 1e12, 4)
    roof["fp64_peak_source"] = ("2 DFMA per SM cycle (ncu sm__inst_executed_pipe_fp64 peak_sustained) x "
                                f"{sms} SMs x {sm_mhz:.0f} MHz (median sampled); live probes: DFMA chains "
                                f"{rates['dfma']:.3g} FMA/s, DMMA {rates.get('dmma', 0):.3g} FMA/s")
    if head == "split":
        ib = issue_bound(f"split_tiles_{dom}_general_stride", M_T * N_S, dk["ms"] * 1e-3, sm_mhz, sms)
        if ib:
            roof["issue"] = ib
    roof["per_form"] = {f: results[f]["per_kernel"] for f in forms}
    roof["pipe_rates_measured"] = {k: float("%.4g" % v) for k, v in rates.items()}

    line = {
        "metric": METRIC, "value": H["value"], "unit": "pair-evals/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": H["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f16x3 split + f32 kernel + f64 sums" if head == "split" else "f64",
        "data": "synthetic: seeded uniform[0,1]^64 pool, N(0,1) weights, random subset / permutation maps",
        "config": {"workload": WORKLOAD, "form": head, "pool": N_POOL, "k": K_DIM, "m": M_T, "n": N_S,
                   "kernels": [k[0] for k in KERNELS],
                   "l2": "flushed between steps (512 MiB memset inside the timed region)",
                   "parallelism": f"replicas x{ws}"},
        "forms": {f: {"value": results[f]["value"], "ms_per_step": results[f]["ms_per_step"]} for f in forms},
        "roofline": roof,
        "gpu_launches": H["gpu_launches"],
        "clocks": clk.summary(),
    }
    if "split" in results and "fp64" in results:
        line["forms"]["split_over_fp64"] = results["split"]["value"] / results["fp64"]["value"]

    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu, err = cpu_baseline_and_error(args, torch, gsks, wl, forms, stream)
        line["cpu_baseline"] = cpu
        line["error"] = err
    if not args.no_e2e:
        line["e2e"] = run_e2e(args, torch, gsks, wl, ws, head)
    if ws == 1 and head == "split":
        line["rhs"] = run_rhs(args, torch, gsks, wl, stream)
    if not args.no_list and ws == 1:
        del wl
        torch.cuda.empty_cache()
        line["list"] = run_list(args, torch, gsks, forms)
    if not args.no_list and ws == 1:
        torch.cuda.empty_cache()
        line["list_local"] = run_list_local(args, torch, gsks)
    if not args.no_configs and ws == 1:
        torch.cuda.empty_cache()
        line["configs"] = run_configs_default(args, torch, gsks)
    return line


def run_rhs(args, torch, gsks, wl, stream, nrhs=4):
    """Several right-hand sides (gsks_dgsks_device_rhs): the Gaussian of the
    step over the same pairs with nrhs interleaved weight columns, split form,
    device-resident; pair-evals/s counts one per pair and right-hand side."""
    g = torch.Generator(device="cuda")
    g.manual_seed(99)
    w = torch.randn(N_S * nrhs, dtype=torch.float64, device="cuda", generator=g)
    u = torch.zeros(M_T * nrhs, dtype=torch.float64, device="cuda")
    name, kt, p, _ = KERNELS[0]
    ker = gsks.make_kernel(kt, **p)
    call = lambda: gsks.dgsks_device_rhs(ker, M_T, N_S, K_DIM, nrhs, u, wl["umap"], wl["X"], wl["X2"], wl["amap"],
                                         wl["X"], wl["X2"], wl["bmap"], w, wl["wmap"],
                                         precision=gsks.GSKS_SPLIT_BF16X3, stream=stream, nxa=N_POOL, nxb=N_POOL)
    for _ in range(max(1, args.warmup)):
        call()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    ts = []
    for _ in range(max(1, args.steps)):
        flush.zero_()
        a = torch.cuda.Event(enable_timing=True); b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        call()
        b.record(stream)
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    ms = statistics.median(ts)
    # one right-hand side through the same entry, for the ratio
    w1 = w[:N_S].contiguous()
    u1 = torch.zeros(M_T, dtype=torch.float64, device="cuda")
    one = lambda: gsks.dgsks_device_rhs(ker, M_T, N_S, K_DIM, 1, u1, wl["umap"], wl["X"], wl["X2"], wl["amap"],
                                        wl["X"], wl["X2"], wl["bmap"], w1, wl["wmap"],
                                        precision=gsks.GSKS_SPLIT_BF16X3, stream=stream, nxa=N_POOL, nxb=N_POOL)
    one()
    t1s = []
    for _ in range(max(1, args.steps)):
        flush.zero_()
        a = torch.cuda.Event(enable_timing=True); b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        one()
        b.record(stream)
        torch.cuda.synchronize()
        t1s.append(a.elapsed_time(b))
    ms1 = statistics.median(t1s)
    out = {"kernel": name, "nrhs": nrhs, "ms": round(ms, 3), "ms_nrhs1": round(ms1, 3),
           "time_ratio_vs_nrhs1": round(ms / ms1, 3), "value": float(M_T) * N_S * nrhs / (ms * 1e-3),
           "unit": "pair-evals/s (per right-hand side)", "form": "split",
           "note": "split form: one sweep, every kernel value formed once and multiplied by the nrhs weight "
                   "columns"}
    # FP64 form on a block of 8192 target rows: nrhs right-hand sides in one
    # pass (each kernel value formed once) against one right-hand side
    mr = 8192
    rows = wl["amap"][:mr]
    urow = torch.arange(mr, dtype=torch.int32, device="cuda")
    ub = torch.zeros(mr * nrhs, dtype=torch.float64, device="cuda")

    def fp64(r):
        gsks.dgsks_device_rhs(ker, mr, N_S, K_DIM, r, ub, urow, wl["X"], wl["X2"], rows, wl["X"], wl["X2"],
                              wl["bmap"], w, wl["wmap"], precision=gsks.GSKS_FP64, stream=stream,
                              nxa=N_POOL, nxb=N_POOL)

    for r in (1, nrhs):
        fp64(r)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True); b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fp64(r)
        b.record(stream)
        torch.cuda.synchronize()
        out[f"fp64_ms_rows{mr}_nrhs{r}"] = round(a.elapsed_time(b), 3)
    out["fp64_note"] = (f"FP64 form, {mr} target rows: {nrhs} right-hand sides in one pass against one; "
                        "w read with stride nrhs in both")
    return out


def run_list_local(args, torch, gsks, k=64, ncl=64, per=2048):
    """Tree-code-like lists (the batched form's intended use: near-field blocks):
    64 clusters (centres U[-10,10]^k, sigma 0.05) of 2048 points, one task per
    cluster (its points against themselves), Gaussian h = 0.2; each task is
    centred and scaled on its own box.  Wall clock around each synchronous
    dgsks_list call, device arrays, both forms."""
    import numpy as np
    rng = np.random.default_rng(5)
    centres = rng.uniform(-10, 10, (ncl, k))
    X = (centres[:, None, :] + 0.05 * rng.standard_normal((ncl, per, k))).reshape(-1, k)
    N = X.shape[0]
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    Xd, wd = dev(X), dev(rng.standard_normal(N))
    idd = dev(np.arange(N, dtype=np.int32))
    offd = dev((np.arange(ncl + 1) * per).astype(np.int32))
    ker = gsks.make_kernel(0, scal=-12.5)
    pairs = float(ncl) * per * per
    out = {"workload": f"{ncl} tasks, each one cluster of {per} points against itself (k={k}, mixture centres "
                       "U[-10,10]^k, sigma 0.05), Gaussian h=0.2", "pairs_per_step": pairs,
           "timing": "wall clock around each synchronous dgsks_list call, device arrays"}
    for form in ("split", "fp64"):
        gsks.set_precision(prec_of(gsks, form))
        u = torch.zeros(N, dtype=torch.float64, device="cuda")
        call = lambda: gsks.dgsks_list(ker, u, offd, idd, offd, idd, Xd, None, Xd, None, wd)
        call()
        torch.cuda.synchronize()
        reps = max(1, args.steps) if form == "split" else 1
        t0 = time.perf_counter()
        for _ in range(reps):
            call()
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / reps
        out[form] = {"value": pairs / dt, "unit": "pair-evals/s", "ms_per_step": dt * 1e3}
    gsks.set_precision(gsks.GSKS_FP64)
    out["split_over_fp64"] = out["split"]["value"] / out["fp64"]["value"]
    return out


def make_list_workload(ntask=LIST_TASKS, seed=4321):
    """Seeded synthetic lists: every task's targets (sources) are a window of a
    random permutation of the pool, so they are distinct within the task."""
    import numpy as np
    rng = np.random.default_rng(seed)
    N = LIST_POOL

    def lists(sz):
        perm = rng.permutation(N).astype(np.int32)
        off = np.concatenate([[0], np.cumsum(sz)]).astype(np.int64)
        tid = np.repeat(np.arange(ntask), sz)
        local = np.arange(off[-1]) - off[tid]
        start = rng.integers(0, N, ntask)
        return off.astype(np.int32), perm[(start[tid] + local) % N].astype(np.int32)

    sa = np.exp(rng.uniform(np.log(32), np.log(4096), ntask)).astype(np.int64)
    sb = np.exp(rng.uniform(np.log(32), np.log(4096), ntask)).astype(np.int64)
    a_off, a_idx = lists(sa)
    b_off, b_idx = lists(sb)
    kinds = rng.integers(0, 3, ntask)
    specs = []
    for t in range(ntask):
        if kinds[t] == 0:
            specs.append((0, dict(scal=-1.0 / (2 * rng.uniform(0.1, 2.0) ** 2))))
        elif kinds[t] == 1:
            specs.append((2, {}))
        else:
            specs.append((1, dict(scal=1.0 / LIST_K, cons=1.0, powe=float(rng.integers(2, 4)))))
    X = rng.random((N, LIST_K))
    w = rng.standard_normal(N)
    return dict(X=X, w=w, a_off=a_off, a_idx=a_idx, b_off=b_off, b_idx=b_idx, specs=specs,
                sa=sa, sb=sb, pairs=float(np.sum(sa * sb)))


def _sub_list(L, tasks):
    import numpy as np
    out = {}
    for side in ("a", "b"):
        off, idx = L[side + "_off"], L[side + "_idx"]
        parts = [idx[off[t]:off[t + 1]] for t in tasks]
        out[side + "_off"] = np.concatenate([[0], np.cumsum([p.size for p in parts])]).astype(np.int32)
        out[side + "_idx"] = np.concatenate(parts).astype(np.int32)
    out["specs"] = [L["specs"][t] for t in tasks]
    out["pairs"] = float(sum(L["sa"][t] * L["sb"][t] for t in tasks))
    return out


def run_list(args, torch, gsks, forms):
    """The batched configuration through dgsks_list with device arrays: wall
    clock around each synchronous call (host planning included); errors of both
    forms on a random subset of tasks against the oracle; the oracle's
    multi-threaded restatement of the reference's list driver as CPU baseline."""
    import numpy as np
    from oracle import oracle as O
    L = make_list_workload()
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    X, w = dev(L["X"]), dev(L["w"])
    out = {"workload": LIST_WORKLOAD, "tasks": LIST_TASKS, "pairs_per_step": L["pairs"],
           "timing": "wall clock around each synchronous dgsks_list call, device-resident arrays; "
                     "host planning, uploads of the plan and the merge included"}

    def call(sub, u, kers):
        gsks.dgsks_list(kers[0], u, dev(sub["a_off"]), dev(sub["a_idx"]), dev(sub["b_off"]), dev(sub["b_idx"]),
                        X, None, X, None, w, kers=kers)

    kers = [gsks.make_kernel(t, **p) for t, p in L["specs"]]
    d_lists = {k: dev(L[k]) for k in ("a_off", "a_idx", "b_off", "b_idx")}
    for form in forms:
        gsks.set_precision(prec_of(gsks, form))
        u = torch.zeros(LIST_POOL, dtype=torch.float64, device="cuda")
        run = lambda: gsks.dgsks_list(kers[0], u, d_lists["a_off"], d_lists["a_idx"], d_lists["b_off"],
                                      d_lists["b_idx"], X, None, X, None, w, kers=kers)
        for _ in range(max(1, args.warmup)):
            run()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            run()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        out[form] = {"value": L["pairs"] * args.steps / dt, "unit": "pair-evals/s",
                     "ms_per_step": dt * 1e3 / args.steps, "gpu_launches": gsks.last_launch_count()}
        # the same lists planned once: every step replays the captured CUDA graph
        plan = gsks.ListPlan(kers[0], d_lists["a_off"], d_lists["a_idx"], d_lists["b_off"], d_lists["b_idx"],
                             LIST_K, LIST_POOL, LIST_POOL, LIST_POOL, LIST_POOL, kers=kers,
                             precision=prec_of(gsks, form), same_pool=True)
        stream = torch.cuda.current_stream()
        for _ in range(max(1, args.warmup)):
            plan.execute(u, X, None, X, None, w, stream=stream)
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True); ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            plan.execute(u, X, None, X, None, w, stream=stream)
        ev1.record(stream)
        torch.cuda.synchronize()
        pt = ev0.elapsed_time(ev1) * 1e-3
        out[form]["planned"] = {"value": L["pairs"] * args.steps / pt, "ms_per_step": pt * 1e3 / args.steps,
                                "timing": "CUDA events around graph replays of gsks_list_plan_execute"}
        assert plan.errors() == 0
        plan.close()
    gsks.set_precision(gsks.GSKS_FP64)
    if "split" in out and "fp64" in out:
        out["split_over_fp64"] = out["split"]["value"] / out["fp64"]["value"]
        out["split_over_fp64_planned"] = out["split"]["planned"]["value"] / out["fp64"]["planned"]["value"]

    # errors on a subset of tasks
    rng = np.random.default_rng(17)
    sub = _sub_list(L, np.sort(rng.choice(LIST_TASKS, 256, replace=False)))
    O.build()
    X2h = O.norms(L["X"])
    okers = [O.make_kernel(t, **p) for t, p in sub["specs"]]
    u_ref = np.zeros(LIST_POOL)
    O.dgsks_list(okers[0], u_ref, sub["a_off"], sub["a_idx"], sub["a_idx"], sub["b_off"], sub["b_idx"],
                 sub["b_idx"], L["X"], X2h, L["X"], X2h, L["w"], kers=okers)
    cond = np.zeros(LIST_POOL)
    for t in range(len(sub["specs"])):
        a0, a1, b0, b1 = sub["a_off"][t], sub["a_off"][t + 1], sub["b_off"][t], sub["b_off"][t + 1]
        amap, bmap = sub["a_idx"][a0:a1], sub["b_idx"][b0:b1]
        _, c = O.rows(okers[t], np.arange(a1 - a0, dtype=np.int32), L["X"], X2h, amap, L["X"], X2h, bmap,
                      L["w"], bmap)
        np.add.at(cond, amap, c)
    named = np.unique(sub["a_idx"])
    err = {"tasks_checked": 256, "pairs_checked": sub["pairs"],
           "metrics": "normwise; cond = max over u entries of |du| / sum |K w| of the positions naming it"}
    skers = [gsks.make_kernel(t, **p) for t, p in sub["specs"]]
    for form in forms:
        gsks.set_precision(prec_of(gsks, form))
        u = torch.zeros(LIST_POOL, dtype=torch.float64, device="cuda")
        call(sub, u, skers)
        torch.cuda.synchronize()
        e = O.errors(u.cpu().numpy()[named], u_ref[named], cond=cond[named])
        err[form] = {k: float("%.3g" % v) for k, v in e.items()}
    gsks.set_precision(gsks.GSKS_FP64)
    out["error"] = err

    # CPU baseline: the oracle's OpenMP list driver on a bounded subset of tasks
    if not args.no_cpu:
        cores = os.cpu_count() or 1
        O.set_threads(cores)
        order = rng.permutation(LIST_TASKS)

        def timed(ntk):
            s2 = _sub_list(L, np.sort(order[:ntk]))
            ok = [O.make_kernel(t, **p) for t, p in s2["specs"]]
            u = np.zeros(LIST_POOL)
            t0 = time.perf_counter()
            O.dgsks_list(ok[0], u, s2["a_off"], s2["a_idx"], s2["a_idx"], s2["b_off"], s2["b_idx"], s2["b_idx"],
                         L["X"], X2h, L["X"], X2h, L["w"], kers=ok, impl="omp")
            return time.perf_counter() - t0, s2["pairs"]

        timed(16)                                              # thread start-up
        t1, p1 = timed(256)
        ntk = int(min(LIST_TASKS, max(256, 256 * args.cpu_seconds / max(t1, 1e-3))))
        t, pairs = timed(ntk)
        out["cpu_baseline"] = {"value": pairs / t, "unit": "pair-evals/s", "cores": cores, "kind": "port",
                               "sample": f"{ntk} random tasks of the list ({pairs:.3g} pairs, {t:.1f} s)",
                               "impl": "oracle_dgsks_list_omp (restated frame/omp_dgsks_list.cpp driver over "
                                       "oracle_dgsks_fused)"}
    return out


def run_e2e(args, torch, gsks, wl, ws, form):
    """The same steps through ks.h dgsks() with host (numpy) arrays."""
    import numpy as np
    h = {k: v.cpu().numpy() for k, v in wl.items()}
    gsks.set_precision(prec_of(gsks, form))
    u = np.zeros(M_T)
    for _, kt, p, _f in KERNELS:   # one warm-up step
        rc = gsks.dgsks_status(gsks.make_kernel(kt, **p), u, h["umap"], h["X"], h["X2"], h["amap"], h["X"],
                               h["X2"], h["bmap"], h["w"], h["wmap"])
        assert rc == 0, gsks.error_string(rc)
    barrier(ws)
    steps = max(1, args.steps)
    t0 = time.perf_counter()
    for _ in range(steps):
        for _, kt, p, _f in KERNELS:
            gsks.dgsks_status(gsks.make_kernel(kt, **p), u, h["umap"], h["X"], h["X2"], h["amap"], h["X"],
                              h["X2"], h["bmap"], h["w"], h["wmap"])
    dt = max_over_ranks(ws, time.perf_counter() - t0)
    gsks.set_precision(gsks.GSKS_FP64)
    # bytes the host path moves per call (copied, or read by the gather kernel):
    # gathered A and B rows, norms, w, u in; u out
    h2d_norm = 8 * (M_T * K_DIM + N_S * K_DIM + M_T + N_S + N_S + M_T)
    h2d_ip = 8 * (M_T * K_DIM + N_S * K_DIM + N_S + M_T)   # the inner-product kernel sends no norms
    return {"value": len(KERNELS) * M_T * N_S * steps * ws / dt, "unit": "pair-evals/s", "form": form,
            "h2d_bytes_per_step": 2 * h2d_norm + h2d_ip, "d2h_bytes_per_step": 8 * M_T * len(KERNELS),
            "path": "ks.h dgsks() with host numpy arrays: " + (
                "rows gathered by a kernel reading the host arrays (the GPU reads pageable host memory)"
                if gsks.host_gather_on_device() else "rows gathered on the host into pinned staging, then copied")}


def cpu_baseline_and_error(args, torch, gsks, wl, forms, stream):
    """CPU port of the reference's fused dgsks on sampled rows x all sources, all
    host cores; the same row sums give each GPU form's error on those rows."""
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
    gpu_u = {}
    for form in forms:
        for name, kt, p, _f in KERNELS:
            u = torch.zeros(M_T, dtype=torch.float64, device="cuda")
            device_call(gsks, wl, kt, p, u, prec_of(gsks, form), stream)
            torch.cuda.synchronize()
            gpu_u[(form, name)] = u.cpu().numpy()
    rng = np.random.default_rng(7)

    def timed(rows):
        t, outs = 0.0, {}
        for name, kt, p, _f in KERNELS:
            amap_s = np.ascontiguousarray(h["amap"][rows])
            u_s = np.zeros(rows.size)
            t0 = time.perf_counter()
            O.dgsks(O.make_kernel(kt, **p), u_s, np.arange(rows.size, dtype=np.int32), h["X"], h["X2"], amap_s,
                    h["X"], h["X2"], h["bmap"], h["w"], h["wmap"], impl="fused")
            t += time.perf_counter() - t0
            outs[name] = u_s
        return t, outs

    timed(np.arange(16, dtype=np.int32))                       # thread start-up
    rows0 = np.sort(rng.choice(M_T, 128, replace=False)).astype(np.int32)
    t0, _ = timed(rows0)
    S = int(min(M_T, max(128, 128 * args.cpu_seconds / max(t0, 1e-3))))
    rows = np.sort(rng.choice(M_T, S, replace=False)).astype(np.int32)
    t, outs = timed(rows)
    pairs = len(KERNELS) * S * N_S
    cpu = {"value": pairs / t, "unit": "pair-evals/s", "cores": cores, "kind": "port",
           "sample": f"{S} random target rows x all {N_S} sources, each of the {len(KERNELS)} kernels "
                     f"({pairs:.3g} pairs, {t:.1f} s)",
           "impl": "oracle_dgsks_fused (C restatement of frame/dgsks.c, OpenMP); the reference's AVX "
                   "micro-kernels do not build on aarch64"}
    err = {"rows_checked": int(S),
           "metrics": "normwise ||du||/||u||; cond = max_i |du_i| / sum_j |K_ij w_j|"}
    for form in forms:
        err[form] = {}
        for name, kt, p, _f in KERNELS:
            _, cond = O.rows(O.make_kernel(kt, **p), rows, h["X"], h["X2"], h["amap"], h["X"], h["X2"],
                             h["bmap"], h["w"], h["wmap"])
            e = O.errors(gpu_u[(form, name)][h["umap"][rows]], outs[name], cond=cond)
            err[form][name] = {k: float("%.3g" % v) for k, v in e.items()}
    return cpu, err


def run_reference(args, ws, rank):
    """The reference's CPU implementation of the path on this host's cores: the
    oracle port of its fused dgsks, bounded sample of target rows per step."""
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
    step(16)
    t0 = time.perf_counter(); step(128); t1 = time.perf_counter() - t0
    budget = min(15.0, 120.0 / max(1, args.steps + args.warmup))   # whole run within a few minutes
    S = int(min(M_T, max(64, 128 * budget / max(t1, 1e-3))))
    for _ in range(args.warmup):
        step(S)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step(S)
    dt = time.perf_counter() - t0
    v = len(KERNELS) * S * N_S * args.steps / dt
    return {"metric": METRIC, "value": v, "unit": "pair-evals/s", "impl": "reference", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: seeded uniform[0,1]^64 pool, N(0,1) weights",
            "config": {"workload": WORKLOAD, "form": "cpu fp64", "sample_rows_per_step": S},
            "cpu_baseline": {"value": v, "unit": "pair-evals/s", "cores": cores, "kind": "port",
                             "sample": f"{S} random target rows x all {N_S} sources x {len(KERNELS)} kernels per step"},
            "e2e": {"value": v, "unit": "pair-evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------------------
# The other configurations of the benchmark specification, each at full size:
# the split form timed over all pairs; the FP64 form timed on a block of target
# rows (its throughput does not depend on m once every SM is busy); errors of
# both on sampled rows against the oracle.
CONFIG_SPECS = {
    "c3": dict(desc="split vs FP64: m=n=131072 points of a 64-component Gaussian mixture (centres U[-10,10]^k, "
                    "sigma 0.05, 1% exact duplicates), targets = sources; Gaussian h=0.2 and polynomial pwr 2",
               m=131072, ks=[3, 8, 32, 128, 512]),
    "c5a": dict(desc="variable-bandwidth Gaussian: m=n=2^20 points uniform[0,1]^8, per-point bandwidth h "
                     "log-uniform in [0.01, 0.5], hi = hj = 1/h (K = exp(-d2 / (2 h_i h_j)))",
                m=1 << 20, ks=[8]),
    "c5b": dict(desc="dense: m=n=262144 points N(0, 1/k), k=1024, polynomial pwr 4 (scal 1, cons 1)",
                m=262144, ks=[1024]),
}


def _config_data(torch, name, k, m, seed):
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    extra = {}
    if name == "c3":
        cent = (torch.rand(64, k, dtype=torch.float64, device="cuda", generator=g) * 20.0 - 10.0)
        lab = torch.randint(0, 64, (m,), device="cuda", generator=g)
        X = cent[lab] + 0.05 * torch.randn(m, k, dtype=torch.float64, device="cuda", generator=g)
        nd = m // 100
        src = torch.randperm(m, device="cuda", generator=g)[:nd]
        dst = torch.randperm(m, device="cuda", generator=g)[:nd]
        X[dst] = X[src]
        kernels = [("gaussian", 0, dict(scal=-12.5)), ("polynomial", 1, dict(scal=1.0 / k, cons=1.0, powe=2.0))]
    elif name == "c5a":
        X = torch.rand(m, k, dtype=torch.float64, device="cuda", generator=g)
        h = torch.exp(torch.rand(m, dtype=torch.float64, device="cuda", generator=g) * (math.log(0.5) - math.log(0.01))
                      + math.log(0.01))
        extra["hinv"] = (1.0 / h).contiguous()
        kernels = [("varbw", 3, {})]
    else:
        X = torch.randn(m, k, dtype=torch.float64, device="cuda", generator=g) / math.sqrt(k)
        kernels = [("polynomial", 1, dict(scal=1.0, cons=1.0, powe=4.0))]
    w = torch.randn(m, dtype=torch.float64, device="cuda", generator=g)
    return X.contiguous(), w, kernels, extra


def config_results(args, torch, gsks, O, cname, ks, clk, flush, steps, warmup):
    """One configuration at full size: per k and kernel, the split form over all
    m*n pairs (median of `steps` calls, L2 flushed before each), the FP64 form
    on a block of target rows x all sources (about 0.3 s), and both forms'
    errors on 256 sampled rows against the oracle.  Both forms are timed
    inside the clock sampler `clk`."""
    import numpy as np
    spec = CONFIG_SPECS[cname]
    m = spec["m"]
    stream = torch.cuda.current_stream()
    peaks = peaks_file()
    tc_peak = peaks.get("bf16_tflops", 1900.0) * 1e12
    results = []
    for k in ks:
        X, w, kernels, extra = _config_data(torch, cname, k, m, 1000 + k)
        X2 = torch.empty(m, dtype=torch.float64, device="cuda")
        gsks.norms_device(X, X2, stream=stream)
        ident = torch.arange(m, dtype=torch.int32, device="cuda")
        for name, kt, p in kernels:
            kp = dict(p)
            if "hinv" in extra:
                kp.update(hi=extra["hinv"], hj=extra["hinv"])
            ker = gsks.make_kernel(kt, **kp)

            def call(u, rows, prec):
                mm = rows.numel()
                gsks.dgsks_device(ker, mm, m, k, u, rows, X, X2, rows, X, X2, ident, w, ident, precision=prec,
                                  stream=stream, nxa=m, nxb=m)

            # split over all pairs
            u = torch.zeros(m, dtype=torch.float64, device="cuda")
            for _ in range(max(1, warmup)):
                call(u, ident, gsks.GSKS_SPLIT_BF16X3)
            u.zero_()
            torch.cuda.synchronize()
            ts = []
            with clk:
                for _ in range(steps):
                    flush.zero_()
                    a = torch.cuda.Event(enable_timing=True); b = torch.cuda.Event(enable_timing=True)
                    a.record(stream)
                    call(u, ident, gsks.GSKS_SPLIT_BF16X3)
                    b.record(stream)
                    torch.cuda.synchronize()
                    ts.append(a.elapsed_time(b))
            t_split = statistics.median(ts) * 1e-3
            pairs = float(m) * m
            u_split = (u / steps).cpu().numpy()
            stats = gsks.split_stats()
            # FP64 on a block of rows sized to about 0.3 s (at least 1024 rows: the
            # plan splits the sources into chunks, so every SM stays busy)
            est = 5.9e11 / (k + 12)
            mr = int(min(m, max(1024, est * 0.3 / m)))
            mr = (mr // 64) * 64
            rows = torch.randperm(m, device="cuda")[:mr].to(torch.int32).sort().values
            uf = torch.zeros(m, dtype=torch.float64, device="cuda")
            call(uf, rows[:64], gsks.GSKS_FP64)
            uf.zero_()
            torch.cuda.synchronize()
            with clk:
                flush.zero_()
                a = torch.cuda.Event(enable_timing=True); b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                call(uf, rows, gsks.GSKS_FP64)
                b.record(stream)
                torch.cuda.synchronize()
            t_fp64 = a.elapsed_time(b) * 1e-3
            fp64_rate = float(mr) * m / t_fp64
            # errors on sampled rows of the FP64 block
            hrows = rows.cpu().numpy()
            rng = np.random.default_rng(k)
            sample = np.sort(rng.choice(hrows, min(256, hrows.size), replace=False)).astype(np.int32)
            Xh = X.cpu().numpy()
            X2h = O.norms(Xh)
            wh = w.cpu().numpy()
            okp = dict(p)
            if "hinv" in extra:
                hh = extra["hinv"].cpu().numpy()
                okp.update(hi=hh, hj=hh)
            idh = np.arange(m, dtype=np.int32)
            ref, cond = O.rows(O.make_kernel(kt, **okp), sample, Xh, X2h, idh, Xh, X2h, idh, wh, idh)
            ufh = uf.cpu().numpy()
            err = {"split": {kk: float("%.3g" % v) for kk, v in O.errors(u_split[sample], ref, cond=cond).items()},
                   "fp64": {kk: float("%.3g" % v) for kk, v in O.errors(ufh[sample], ref, cond=cond).items()}}
            alg = 2.0 * pairs * k
            sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
            p64 = fp64_peak(sms, clk.summary().get("sm_mhz") or 2070.0)
            results.append({"k": k, "kernel": name, "pairs": pairs,
                            "split": {"value": pairs / t_split, "ms": round(t_split * 1e3, 3),
                                      "alg_tflops": round(alg / t_split / 1e12, 2),
                                      "frac_alg_tensor": round(alg / tc_peak / t_split, 4),
                                      "rechecked_pairs": stats["rechecked_pairs"],
                                      "rescued_rows": stats["rescued_rows"]},
                            "fp64": {"value": fp64_rate, "rows_timed": mr, "ms": round(t_fp64 * 1e3, 2),
                                     "frac_rank_k": round(2.0 * k * fp64_rate / p64, 4)},
                            "split_over_fp64": (pairs / t_split) / fp64_rate,
                            "error": err, "rows_checked": int(sample.size)})
            del u, uf
        del X, X2, w, ident
        torch.cuda.empty_cache()
    return results


CONFIG_TIMING = ("split: CUDA events per call over all m*n pairs, median of the timed steps, L2 flushed before "
                 "each; fp64: one call over a block of target rows x all sources, L2 flushed before it")


def run_config(args):
    import torch
    from ks_gb300 import build as B
    if not os.path.exists(B.LIB):
        B.build()
    from ks_gb300 import gsks
    from oracle import oracle as O
    torch.cuda.set_device(0)
    spec = CONFIG_SPECS[args.config]
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    O.build()
    O.set_threads(os.cpu_count() or 1)
    clk = ClockSampler(0)
    results = config_results(args, torch, gsks, O, args.config, spec["ks"], clk, flush, args.steps, args.warmup)
    line = {"metric": METRIC, "unit": "pair-evals/s", "config": {"workload": spec["desc"], "name": args.config},
            "steps": args.steps, "warmup": args.warmup, "data": "synthetic, seeded (torch generator on the device)",
            "timing": CONFIG_TIMING, "results": results, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


# The other configurations carried by the default line (key "configs"): the
# mixture at its smallest and largest k, the variable-bandwidth and the dense
# configuration, all at full size.
DEFAULT_CONFIGS = [("c3", [3, 512]), ("c5a", [8]), ("c5b", [1024])]


def run_configs_default(args, torch, gsks):
    from oracle import oracle as O
    O.build()
    O.set_threads(os.cpu_count() or 1)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    clk = ClockSampler(0)
    steps = max(1, min(args.steps, 3))
    out = {"timing": CONFIG_TIMING, "steps": steps, "warmup": 1,
           "data": "synthetic, seeded (torch generator on the device)"}
    for cname, ks in DEFAULT_CONFIGS:
        out[cname] = {"workload": CONFIG_SPECS[cname]["desc"],
                      "results": config_results(args, torch, gsks, O, cname, ks, clk, flush, steps, 1)}
    out["clocks"] = clk.summary()
    return out


def main():
    args = parse()
    if args.case:
        run_case(args)
        return
    if args.config:
        run_config(args)
        return
    if args.impl == "reference":
        ws = int(os.environ.get("WORLD_SIZE", "1")); rank = int(os.environ.get("RANK", "0"))
        line = run_reference(args, ws, rank)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    ws, rank, local = dist_setup()
    line = run_ours(args, ws, rank, local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
