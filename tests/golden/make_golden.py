"""Generates the golden vectors in tests/golden/ from the reference itself.

Runs the reference library compiled from its own sources (oracle/_ref, built
by oracle/build_ref.sh) on seeded inputs and stores inputs and outputs:
  u_ref    -- reference dgsks_ref   (frame/dgsks_ref.c:94-535)
  u_dgsks  -- reference dgsks       (frame/dgsks.c:367-776, Sandy Bridge micro-kernels)
  u_list   -- reference omp_dgsks_list (frame/omp_dgsks_list.cpp:297-420), list cases
  powe/scal after the call (Laplace overwrites them, frame/dgsks_ref.c:146-148).
Inputs are drawn with numpy default_rng(seed); the seeds are in CASES.
Run from the repository root:  python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

# name, kernel type, params, pool N, k, m, n, maps, data, seed
CASES = [
    ("gauss_identity", O.KS_GAUSSIAN, dict(scal=-0.5), 256, 16, 256, 256, "identity", "ref01", 1),
    ("gauss_general", O.KS_GAUSSIAN, dict(scal=-2.0), 300, 16, 160, 120, "general", "unif", 2),
    ("varbw_general", O.KS_GAUSSIAN_VAR_BANDWIDTH, {}, 300, 16, 150, 130, "general", "ref01", 3),
    ("poly4_general", O.KS_POLYNOMIAL, dict(powe=4.0, scal=0.1, cons=0.1), 300, 16, 140, 150, "general", "ref01", 4),
    ("poly3_general", O.KS_POLYNOMIAL, dict(powe=3.0, scal=1.0 / 16, cons=1.0), 300, 16, 150, 140, "general", "unif", 5),
    ("poly2_general", O.KS_POLYNOMIAL, dict(powe=2.0, scal=0.5, cons=-0.25), 300, 16, 100, 90, "general", "unif", 6),
    ("laplace_general", O.KS_LAPLACE, {}, 300, 16, 150, 150, "general", "ref01", 7),
    ("laplace_k3", O.KS_LAPLACE, {}, 300, 3, 120, 110, "general", "unif", 8),
    ("laplace_k37", O.KS_LAPLACE, {}, 200, 37, 100, 90, "general", "unif", 9),
    ("tanh_general", O.KS_TANH, dict(scal=0.1, cons=0.1), 300, 16, 130, 150, "general", "ref01", 10),
    ("quartic_general", O.KS_QUARTIC, {}, 300, 16, 150, 120, "general", "ref01", 11),
    ("multiquad_general", O.KS_MULTIQUADRATIC, dict(cons=1.0), 300, 16, 120, 150, "general", "ref01", 12),
    ("epan_general", O.KS_EPANECHNIKOV, {}, 300, 16, 150, 110, "general", "ref01", 13),
    ("gauss_k1", O.KS_GAUSSIAN, dict(scal=-0.5), 200, 1, 100, 100, "general", "unif", 14),
    ("gauss_m1n1", O.KS_GAUSSIAN, dict(scal=-0.5), 50, 8, 1, 1, "general", "unif", 15),
    ("gauss_m1", O.KS_GAUSSIAN, dict(scal=-0.5), 400, 8, 1, 333, "general", "unif", 16),
    ("gauss_n1", O.KS_GAUSSIAN, dict(scal=-0.5), 400, 8, 333, 1, "general", "unif", 17),
    ("gauss_tails", O.KS_GAUSSIAN, dict(scal=-0.5), 300, 13, 67, 33, "general", "unif", 18),
    ("gauss_k300", O.KS_GAUSSIAN, dict(scal=-0.01), 96, 300, 80, 70, "general", "unif", 19),
]

LIST_CASES = [
    # name, type, params, pool N, k, ntask, size range, seed
    ("list_gauss", O.KS_GAUSSIAN, dict(scal=-0.5), 600, 8, 12, (20, 120), 31),
    ("list_laplace", O.KS_LAPLACE, {}, 500, 6, 9, (10, 90), 32),
]


def points(rng, N, k, kind):
    if kind == "ref01":  # the reference drivers' rand()%100/1000 grid (test/test_dgsks.c:167-171)
        return np.floor(rng.random((N, k)) * 100.0) / 1000.0
    return rng.random((N, k))


def make_case(name, ktype, params, N, k, m, n, maps, data, seed):
    rng = np.random.default_rng(seed)
    X = points(rng, N, k, data)
    X2 = O.norms(X)
    w = rng.standard_normal(N)
    u0 = rng.standard_normal(N)
    if maps == "identity":
        amap = np.arange(m, dtype=np.int32); bmap = np.arange(n, dtype=np.int32)
        umap = amap.copy(); wmap = bmap.copy()
    else:
        amap = rng.choice(N, m, replace=False).astype(np.int32)
        bmap = rng.choice(N, n, replace=False).astype(np.int32)
        umap = rng.permutation(N)[:m].astype(np.int32)
        wmap = rng.permutation(N)[:n].astype(np.int32)
    hi = np.zeros(1)
    if ktype == O.KS_GAUSSIAN_VAR_BANDWIDTH:
        # bandwidth of the reference driver (test/test_dgsks.c:199-207)
        s = 1.0 + 0.5 / (1.0 + np.exp(-X2))
        hi = -1.0 / (2.0 * s * s)
    out = dict(X=X, X2=X2, w=w, u0=u0, amap=amap, bmap=bmap, umap=umap, wmap=wmap, hi=hi)
    for impl, key in (("reference", "u_ref"), ("reference_dgsks", "u_dgsks")):
        ker = O.make_kernel(ktype, **params, **({"hi": hi, "hj": hi} if hi.size > 1 else {}))
        u = u0.copy()
        O.dgsks(ker, u, umap, X, X2, amap, X, X2, bmap, w, wmap, impl=impl)
        out[key] = u
        out["powe_after"] = np.array(ker.powe); out["scal_after"] = np.array(ker.scal)
    meta = dict(type=ktype, params=params, N=N, k=k, m=m, n=n, maps=maps, data=data, seed=seed)
    return out, meta


def make_list_case(name, ktype, params, N, k, ntask, rng_sz, seed):
    rng = np.random.default_rng(seed)
    X = points(rng, N, k, "ref01")
    X2 = O.norms(X)
    w = rng.standard_normal(N)
    u0 = np.zeros(N)
    a_sz = rng.integers(rng_sz[0], rng_sz[1], ntask); b_sz = rng.integers(rng_sz[0], rng_sz[1], ntask)
    a_idx = np.concatenate([rng.permutation(N)[:s] for s in a_sz]).astype(np.int32)
    b_idx = np.concatenate([rng.permutation(N)[:s] for s in b_sz]).astype(np.int32)
    a_off = np.concatenate([[0], np.cumsum(a_sz)]).astype(np.int32)
    b_off = np.concatenate([[0], np.cumsum(b_sz)]).astype(np.int32)
    out = dict(X=X, X2=X2, w=w, u0=u0, a_off=a_off, a_idx=a_idx, b_off=b_off, b_idx=b_idx)
    ker = O.make_kernel(ktype, **params)
    u = u0.copy()
    O.dgsks_list(ker, u, a_off, a_idx, a_idx, b_off, b_idx, b_idx, X, X2, X, X2, w, impl="reference")
    out["u_list"] = u
    # per-task dgsks_ref loop, as test/test_dgsks_list.cpp:213-230 checks it
    u = u0.copy()
    for t in range(ntask):
        ker = O.make_kernel(ktype, **params)
        sa, sb = slice(a_off[t], a_off[t + 1]), slice(b_off[t], b_off[t + 1])
        O.dgsks(ker, u, a_idx[sa].copy(), X, X2, a_idx[sa].copy(), X, X2, b_idx[sb].copy(), w,
                b_idx[sb].copy(), impl="reference")
    out["u_ref"] = u
    meta = dict(type=ktype, params=params, N=N, k=k, ntask=ntask, sizes=list(rng_sz), seed=seed)
    return out, meta


def main():
    if not O.reference_available():
        raise SystemExit("reference not built: run oracle/build_ref.sh")
    manifest = {}
    for c in CASES:
        arrs, meta = make_case(*c)
        np.savez_compressed(os.path.join(OUT, c[0] + ".npz"), **arrs)
        manifest[c[0]] = meta
    for c in LIST_CASES:
        arrs, meta = make_list_case(*c)
        np.savez_compressed(os.path.join(OUT, c[0] + ".npz"), **arrs)
        manifest[c[0]] = meta
    with open(os.path.join(OUT, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
    print("wrote", len(manifest), "cases")


if __name__ == "__main__":
    main()
