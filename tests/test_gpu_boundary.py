"""The drop-in boundary against the oracle: every entry a reference caller binds.

* all five C++ list signatures of omp_dgsks_list.hpp (frame/omp_dgsks_list.cpp:
  55-294 wrappers, 297-420 core), called from a g++-built program;
* the ctypes entries dgsks_wrapper / dgsks_ref_wrapper (frame/dgsks.c:783-826,
  frame/dgsks_ref.c:537-580) with a polynomial cons != 0, which the reference's
  Python binding drops (python/gsks.py:53-54) and these forward;
* the reference-style Python functions gsks.dgsks / gsks.dgsks_ref
  (python/gsks.py:18-199) for all eight kernel type names.

FP64 form, tolerance 1e-12 on the added part of u (normwise), as the other
FP64 parity tests."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _compile(src, out, cxx):
    inc = os.path.join(ROOT, "include")
    lib = os.path.join(ROOT, "ks_gb300", "lib")
    cmd = [cxx, "-O1", "-I" + inc, src, "-o", out, "-L" + lib, "-lgsks", "-Wl,-rpath," + lib, "-lm"]
    subprocess.run(cmd, check=True, capture_output=True)


def _close(got, ref, u0, tol=TOL):
    du, dr = got - u0, ref - u0
    assert np.abs(dr).max() > 0
    err = np.linalg.norm(du - dr) / np.linalg.norm(dr)
    assert err <= tol, err
    assert np.array_equal(got[dr == 0], u0[dr == 0])


@pytest.mark.parametrize("kern", [(0, -0.5, 0.0, 1.0), (1, 1.0 / 7, 0.5, 3.0), (2, 0.0, 0.0, 1.0)],
                         ids=["gaussian", "polynomial", "laplace"])
def test_cpp_list_signatures_match_oracle(gpu, oracle_mod, tmp_path, kern):
    O = oracle_mod
    rng = np.random.default_rng(61 + kern[0])
    N, k, ntask = 3000, 7, 9
    XA = rng.random((N, k))
    XB = rng.random((N, k)) * 1.1
    w = rng.standard_normal(N)
    u0 = rng.standard_normal(N)
    sa = rng.integers(0, 400, ntask); sb = rng.integers(0, 300, ntask)
    sa[2] = 0; sb[5] = 0                                        # empty tasks
    a_idx = np.concatenate([rng.permutation(N)[:s] for s in sa]).astype(np.int32)
    u_idx = np.concatenate([rng.permutation(N)[:s] for s in sa]).astype(np.int32)
    b_idx = np.concatenate([rng.permutation(N)[:s] for s in sb]).astype(np.int32)
    w_idx = rng.integers(0, N, b_idx.size).astype(np.int32)
    a_off = np.concatenate([[0], np.cumsum(sa)]).astype(np.int32)
    b_off = np.concatenate([[0], np.cumsum(sb)]).astype(np.int32)

    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(fin, "wb") as f:
        np.array([N, N, k, ntask, N, N], np.int32).tofile(f)
        np.array(kern, np.float64).tofile(f)
        for a in (XA, XB, w, u0):
            np.ascontiguousarray(a, np.float64).tofile(f)
        for a in (a_off, a_idx, u_idx, b_off, b_idx, w_idx):
            a.astype(np.int32).tofile(f)
    exe = str(tmp_path / "list_signatures")
    _compile(os.path.join(ROOT, "tests", "c", "list_signatures.cpp"), exe, "g++")
    run = subprocess.run([exe, fin, fout], capture_output=True, text=True)
    assert run.returncode == 0, (run.returncode, run.stderr)
    got = np.fromfile(fout, np.float64).reshape(5, N)

    XA2, XB2 = O.norms(XA), O.norms(XB)
    ker = lambda: O.make_kernel(int(kern[0]), scal=kern[1], cons=kern[2], powe=kern[3])
    expect = {
        0: (a_idx, XB, XB2),     # unsymmetric: ulist = alist, sources from XB
        1: (a_idx, XA, XA2),     # symmetric: ulist = alist, sources from XA
        2: (u_idx, XB, XB2),     # separated u, unsymmetric
        3: (u_idx, XA, XA2),     # separated u, symmetric
        4: (u_idx, XB, XB2),     # the core signature, norms from the caller
    }
    for form, (ui, Xs, Xs2) in expect.items():
        ref = u0.copy()
        O.dgsks_list(ker(), ref, a_off, a_idx, ui, b_off, b_idx, w_idx, XA, XA2, Xs, Xs2, w)
        _close(got[form], ref, u0)


def _single_case(seed, N=900, k=5, m=300, n=400, scale=1.0):
    rng = np.random.default_rng(seed)
    X = rng.random((N, k)) * scale
    w = rng.standard_normal(N)
    u0 = rng.standard_normal(N)
    amap = rng.choice(N, m, replace=False).astype(np.int32)
    bmap = rng.choice(N, n, replace=False).astype(np.int32)
    umap = rng.permutation(N)[:m].astype(np.int32)
    wmap = rng.permutation(N)[:n].astype(np.int32)
    return X, w, u0, amap, bmap, umap, wmap


@pytest.mark.parametrize("entry", ["dgsks_wrapper", "dgsks_ref_wrapper"])
def test_ctypes_wrappers_forward_cons(gpu, oracle_mod, entry):
    from ks_gb300 import gsks
    O = oracle_mod
    lib = gsks.load()
    X, w, u0, amap, bmap, umap, wmap = _single_case(71)
    X2 = O.norms(X)
    m, n, k = amap.size, bmap.size, X.shape[1]
    scal, cons, powe = 0.3, 0.7, 3.0
    u = u0.copy()
    p = lambda a: C.c_void_p(a.ctypes.data)
    h = np.zeros(1)
    fn = getattr(lib, entry)
    fn.restype = None
    fn(C.c_int(m), C.c_int(n), C.c_int(k), p(u), p(umap), p(X), p(X2), p(amap), p(X), p(X2), p(bmap), p(w), p(wmap),
       C.c_int(1), C.c_double(scal), C.c_double(cons), C.c_double(powe), p(h))
    assert gsks.last_error() == 0
    ref = u0.copy()
    O.dgsks(O.make_kernel(1, scal=scal, cons=cons, powe=powe), ref, umap, X, X2, amap, X, X2, bmap, w, wmap)
    _close(u, ref, u0)
    # the test tells the two apart: without cons the result differs at O(1)
    ref0 = u0.copy()
    O.dgsks(O.make_kernel(1, scal=scal, cons=0.0, powe=powe), ref0, umap, X, X2, amap, X, X2, bmap, w, wmap)
    assert np.linalg.norm(u - ref0) > 1e-3 * np.linalg.norm(ref0 - u0)


# (type name of python/gsks.py, ks_type, options, coordinate scale)
NAMED = [
    ("Gaussian", 0, dict(scal=-0.7), 1.0),
    ("Polynomial", 1, dict(scal=0.4, cons=0.6, powe=3.0), 1.0),
    ("Laplace", 2, dict(), 1.0),
    ("Variable_Bandwidth", 3, dict(), 1.0),
    ("Tanh", 4, dict(scal=0.5, cons=-0.2), 1.0),
    ("Quartic", 5, dict(), 0.4),
    ("Multiquadratic", 6, dict(cons=0.9), 1.0),
    ("Epanechnikov", 7, dict(), 0.4),
]


@pytest.mark.parametrize("name,ktype,opts,scale", NAMED, ids=[x[0] for x in NAMED])
@pytest.mark.parametrize("fn", ["dgsks", "dgsks_ref"])
def test_reference_style_binding_all_types(gpu, oracle_mod, name, ktype, opts, scale, fn):
    from ks_gb300 import gsks
    O = oracle_mod
    X, w, u0, amap, bmap, umap, wmap = _single_case(80 + ktype, scale=scale)
    X2 = O.norms(X)
    d = X.shape[1]
    options = dict(opts)
    okw = dict(opts)
    if ktype == 3:
        h = np.exp(np.random.default_rng(5).uniform(np.log(1.0), np.log(20.0), X.shape[0]))
        options["h"] = h
        okw.update(hi=h, hj=h)
    u = u0.copy()
    gsks.set_precision(gsks.GSKS_FP64)
    getattr(gsks, fn)(d, u, umap, X, X2, amap, X, X2, bmap, w, wmap, type=name, **options)
    ref = u0.copy()
    O.dgsks(O.make_kernel(ktype, **okw), ref, umap, X, X2, amap, X, X2, bmap, w, wmap)
    _close(u, ref, u0)
