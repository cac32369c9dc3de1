"""dgsks_list (persistent batched launch) and the C/C++ link surface on the GPU."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_manifest, load_golden

pytestmark = pytest.mark.gpu

MANIFEST = golden_manifest()
LISTS = sorted(k for k, v in MANIFEST.items() if "ntask" in v)


@pytest.mark.parametrize("name", LISTS)
def test_list_host_matches_reference(gpu, oracle_mod, name):
    from ks_gb300 import gsks
    meta, g = MANIFEST[name], load_golden(name)
    u = g["u0"].copy()
    gsks.dgsks_list(gsks.make_kernel(meta["type"], **meta["params"]), u, g["a_off"], g["a_idx"], g["b_off"],
                    g["b_idx"], g["X"], g["X2"], g["X"], g["X2"], g["w"])
    err = oracle_mod.errors(u, g["u_list"])
    assert err["normwise"] <= 1e-12, err
    assert oracle_mod.errors(u, g["u_ref"])["normwise"] <= 1e-12


@pytest.mark.parametrize("name", LISTS)
def test_list_device_matches_reference(gpu, oracle_mod, name):
    from ks_gb300 import gsks
    torch = gpu
    meta, g = MANIFEST[name], load_golden(name)
    d = {k: torch.from_numpy(v).cuda() for k, v in g.items()}
    u = d["u0"].clone()
    gsks.dgsks_list(gsks.make_kernel(meta["type"], **meta["params"]), u, d["a_off"], d["a_idx"], d["b_off"],
                    d["b_idx"], d["X"], None, d["X"], None, d["w"])   # norms computed on the device
    assert oracle_mod.errors(u.cpu().numpy(), g["u_list"])["normwise"] <= 1e-12


def _lists(rng, N, ntask, lo, hi):
    a_sz = rng.integers(lo, hi, ntask); b_sz = rng.integers(lo, hi, ntask)
    a_idx = np.concatenate([rng.permutation(N)[:s] for s in a_sz]).astype(np.int32)
    b_idx = np.concatenate([rng.permutation(N)[:s] for s in b_sz]).astype(np.int32)
    a_off = np.concatenate([[0], np.cumsum(a_sz)]).astype(np.int32)
    b_off = np.concatenate([[0], np.cumsum(b_sz)]).astype(np.int32)
    return a_off, a_idx, b_off, b_idx


def test_list_per_task_kernels_and_separate_maps(gpu, oracle_mod):
    """Per-task descriptors (Gaussian / Laplace / polynomial), separate u and w maps,
    uneven sizes including empty tasks, against the oracle's list restatement."""
    from ks_gb300 import gsks
    O = oracle_mod
    rng = np.random.default_rng(5)
    N, k, ntask = 3000, 16, 40
    X = rng.random((N, k)); X2 = O.norms(X); w = rng.standard_normal(N)
    a_off, a_idx, b_off, b_idx = _lists(rng, N, ntask, 0, 400)
    # u entries are distinct within a task and shared across tasks
    u_idx = np.concatenate([rng.permutation(N)[:a_off[t + 1] - a_off[t]] for t in range(ntask)]).astype(np.int32)
    w_idx = rng.integers(0, N, b_idx.size).astype(np.int32)
    specs = []
    for t in range(ntask):
        c = t % 3
        specs.append((0, dict(scal=-1.0 / (2 * rng.uniform(0.1, 2) ** 2))) if c == 0 else
                     (2, {}) if c == 1 else (1, dict(scal=1.0 / k, cons=1.0, powe=float(2 + t % 2))))
    kers_o = [O.make_kernel(t, **p) for t, p in specs]
    kers_g = [gsks.make_kernel(t, **p) for t, p in specs]
    u_ref = np.zeros(N)
    # every u entry may be named by several positions: oracle per task, in task order
    O.dgsks_list(kers_o[0], u_ref, a_off, a_idx, u_idx, b_off, b_idx, w_idx, X, X2, X, X2, w, kers=kers_o)
    u = np.zeros(N)
    gsks.dgsks_list(kers_g[0], u, a_off, a_idx, b_off, b_idx, X, X2, X, X2, w, u_idx=u_idx, w_idx=w_idx,
                    kers=kers_g)
    assert O.errors(u, u_ref)["normwise"] <= 1e-12
    # deterministic across runs
    u2 = np.zeros(N)
    gsks.dgsks_list(kers_g[0], u2, a_off, a_idx, b_off, b_idx, X, X2, X, X2, w, u_idx=u_idx, w_idx=w_idx,
                    kers=kers_g)
    assert np.array_equal(u, u2)


def _compile(src, out, cxx):
    inc = os.path.join(ROOT, "include")
    lib = os.path.join(ROOT, "ks_gb300", "lib")
    cmd = [cxx, "-O1", "-I" + inc, src, "-o", out, "-L" + lib, "-lgsks", "-Wl,-rpath," + lib, "-lm"]
    subprocess.run(cmd, check=True, capture_output=True)


def test_c_caller_links_unchanged(gpu, oracle_mod, tmp_path):
    exe = str(tmp_path / "link_dgsks")
    _compile(os.path.join(ROOT, "tests", "c", "link_dgsks.c"), exe, "gcc")
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    vals = np.array(out, dtype=np.float64).reshape(-1, 2)
    assert np.abs(vals[:, 0]).max() > 0
    # the program's inputs (its LCG and formulas), then the oracle's dgsks_ref
    O = oracle_mod
    N, K, M, NS = 300, 9, 120, 100
    X = np.empty(N * K)
    s = 12345
    for i in range(N * K):
        s = (s * 1103515245 + 12345) & 0xFFFFFFFF
        X[i] = ((s >> 8) % 1000) / 1000.0
    X = X.reshape(N, K)
    X2 = O.norms(X)
    w = ((np.arange(N) * 37) % 17) / 17.0 - 0.5
    amap = ((np.arange(M) * 7) % N).astype(np.int32)
    umap = ((np.arange(M) * 11) % N).astype(np.int32)
    bmap = ((np.arange(NS) * 13 + 5) % N).astype(np.int32)
    wmap = ((np.arange(NS) * 3 + 1) % N).astype(np.int32)
    u_ref = np.zeros(N)
    O.dgsks(O.make_kernel(0, scal=-0.5), u_ref, umap, X, X2, amap, X, X2, bmap, w, wmap)
    for col in range(2):   # dgsks() and dgsks_ref() as the program linked them
        assert np.linalg.norm(vals[:, col] - u_ref) <= 1e-12 * np.linalg.norm(u_ref), col


def test_cpp_list_caller_links_unchanged(gpu, oracle_mod, tmp_path):
    exe = str(tmp_path / "link_list")
    _compile(os.path.join(ROOT, "tests", "c", "link_list.cpp"), exe, "g++")
    u = np.array(subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split(), dtype=np.float64)
    # same lists through the oracle
    O = oracle_mod
    nx, k, ntask = 500, 6, 7
    X = np.empty(nx * k)
    s = 777
    for i in range(nx * k):
        s = (s * 1664525 + 1013904223) & 0xFFFFFFFF
        X[i] = ((s >> 9) % 100) / 1000.0
    X = X.reshape(nx, k); X2 = O.norms(X)
    w = 1.0 + 0.001 * (np.arange(nx) % 13)
    a = [[(i * 7 + t * 31) % nx for i in range(30 + 17 * t)] for t in range(ntask)]
    b = [[(j * 3 + t * 5) % nx for j in range(25 + 11 * t)] for t in range(ntask)]
    a_off = np.array([0] + list(np.cumsum([len(x) for x in a])), np.int32)
    b_off = np.array([0] + list(np.cumsum([len(x) for x in b])), np.int32)
    a_idx = np.array(sum(a, []), np.int32); b_idx = np.array(sum(b, []), np.int32)
    u_ref = np.zeros(nx)
    O.dgsks_list(O.make_kernel(0, scal=-0.5), u_ref, a_off, a_idx, a_idx, b_off, b_idx, b_idx, X, X2, X, X2, w)
    assert O.errors(u, u_ref)["normwise"] <= 1e-12
