"""ctypes front end of the CPU oracle (test infrastructure only).

Loads ``oracle/_build/liboracle.so`` -- the C restatement in
``oracle/gsks_oracle.c`` -- and, where it was built on this machine,
``oracle/_ref/libgsks_ref.so`` -- the reference library compiled from its own
sources by ``oracle/build_ref.sh``.  Only the tests, ``__graft_entry__.smoke``
and the CPU legs of ``bench.py`` import this module; the product library never
does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libgsks_ref.so")
REF_SHIM_SO = os.path.join(HERE, "_ref", "libref_list_shim.so")

# ks_type values (reference include/ks.h:49-58)
KS_GAUSSIAN, KS_POLYNOMIAL, KS_LAPLACE, KS_GAUSSIAN_VAR_BANDWIDTH = 0, 1, 2, 3
KS_TANH, KS_QUARTIC, KS_MULTIQUADRATIC, KS_EPANECHNIKOV = 4, 5, 6, 7
KERNEL_NAMES = {
    "gaussian": KS_GAUSSIAN, "polynomial": KS_POLYNOMIAL, "laplace": KS_LAPLACE,
    "var_bandwidth": KS_GAUSSIAN_VAR_BANDWIDTH, "tanh": KS_TANH,
    "quartic": KS_QUARTIC, "multiquadratic": KS_MULTIQUADRATIC,
    "epanechnikov": KS_EPANECHNIKOV,
}


class KsT(C.Structure):
    """Layout of ks_t (reference include/ks.h:60-71)."""
    _fields_ = [("type", C.c_int), ("powe", C.c_double), ("scal", C.c_double),
                ("cons", C.c_double), ("hi", C.c_void_p), ("hj", C.c_void_p),
                ("h", C.c_void_p)]


def make_kernel(ktype: int, scal=0.0, cons=0.0, powe=1.0, hi=None, hj=None) -> KsT:
    ker = KsT()
    ker.type, ker.scal, ker.cons, ker.powe = int(ktype), float(scal), float(cons), float(powe)
    ker.hi = hi.ctypes.data if hi is not None else None
    ker.hj = hj.ctypes.data if hj is not None else None
    ker.h = None
    return ker


def build(quiet: bool = True) -> None:
    """Compile liboracle.so with the portable Makefile (either machine)."""
    out = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)


def build_reference() -> bool:
    """Compile the reference into oracle/_ref when its sources are present.

    The recipe (build_ref.sh) locates the sources (variable GSKS_REFERENCE)
    and exits non-zero when they are absent, as on machines without them."""
    out = subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")],
                         capture_output=True, text=True)
    return out.returncode == 0


_LIBS: dict = {}


def _lib(which: str):
    if which in _LIBS:
        return _LIBS[which]
    path = {"oracle": ORACLE_SO, "reference": REF_SO, "shim": REF_SHIM_SO}[which]
    if which == "oracle" and not os.path.exists(path):
        build()
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    mode = C.RTLD_GLOBAL if which == "reference" else C.RTLD_LOCAL
    lib = C.CDLL(path, mode=mode)
    _LIBS[which] = lib
    return lib


def reference_available() -> bool:
    return os.path.exists(REF_SO)


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else C.c_void_p(None)


def _check(arrs):
    for a in arrs:
        assert a.flags["C_CONTIGUOUS"], "arrays must be C-contiguous"


def set_threads(nt: int) -> None:
    _lib("oracle").oracle_set_threads(C.c_int(nt))


def get_threads() -> int:
    return int(_lib("oracle").oracle_get_threads())


def norms(X: np.ndarray) -> np.ndarray:
    N, k = X.shape
    X2 = np.empty(N, dtype=np.float64)
    _lib("oracle").oracle_norms(C.c_int(N), C.c_int(k), _p(X), _p(X2))
    return X2


def dgsks(ker: KsT, u, umap, XA, XA2, amap, XB, XB2, bmap, w, wmap, impl="oracle") -> int:
    """In-place kernel summation into u.

    impl: "oracle" (restated dgsks_ref), "fused" (restated blocked dgsks, the
    CPU baseline), "reference" (reference dgsks_ref) or "reference_dgsks"
    (reference fused dgsks, single-threaded build)."""
    _check([u, umap, XA, amap, XB, bmap, w, wmap])
    m, n = int(amap.size), int(bmap.size)
    k = int(XA.shape[1]) if XA.ndim == 2 else int(XA.size // max(1, XA2.size))
    args = (C.byref(ker), C.c_int(m), C.c_int(n), C.c_int(k), _p(u), _p(umap),
            _p(XA), _p(XA2), _p(amap), _p(XB), _p(XB2), _p(bmap), _p(w), _p(wmap))
    if impl == "oracle":
        return int(_lib("oracle").oracle_dgsks_ref(*args))
    if impl == "fused":
        return int(_lib("oracle").oracle_dgsks_fused(*args))
    if impl == "reference":
        _lib("reference").dgsks_ref(*args)
        return 0
    if impl == "reference_dgsks":
        _lib("reference").dgsks(*args)
        return 0
    raise ValueError(impl)


def rows(ker: KsT, rows_idx, XA, XA2, amap, XB, XB2, bmap, w, wmap):
    """(sum_j K w, sum_j |K w|) for target positions rows_idx (Neumaier sums)."""
    rows_idx = np.ascontiguousarray(rows_idx, dtype=np.int32)
    s = np.zeros(rows_idx.size, dtype=np.float64)
    a = np.zeros(rows_idx.size, dtype=np.float64)
    k = int(XA.shape[1])
    rc = _lib("oracle").oracle_rows(
        C.byref(ker), C.c_int(rows_idx.size), _p(rows_idx), C.c_int(bmap.size), C.c_int(k),
        _p(XA), _p(XA2), _p(amap), _p(XB), _p(XB2), _p(bmap), _p(w), _p(wmap), _p(s), _p(a))
    if rc:
        raise RuntimeError(f"oracle_rows rc={rc}")
    return s, a


def dgsks_list(ker: KsT, u, a_off, a_idx, u_idx, b_off, b_idx, w_idx, XA, XA2, XB, XB2, w,
               kers=None, impl="oracle") -> int:
    """Batched evaluation over CSR task lists, accumulating into u.

    impl: "oracle" (serial restatement), "omp" (multi-threaded restatement of
    the reference's OpenMP list driver, the CPU baseline) or "reference"."""
    k = int(XA.shape[1])
    ntask = int(a_off.size - 1)
    if impl == "oracle":
        karr = None
        if kers is not None:
            karr = (KsT * ntask)(*kers)
        return int(_lib("oracle").oracle_dgsks_list(
            C.byref(ker), karr, C.c_int(ntask), C.c_int(k), _p(u),
            _p(a_off), _p(a_idx), _p(u_idx), _p(b_off), _p(b_idx), _p(w_idx),
            _p(XA), _p(XA2), _p(XB), _p(XB2), _p(w)))
    if impl == "omp":
        karr = None
        if kers is not None:
            karr = (KsT * ntask)(*kers)
        return int(_lib("oracle").oracle_dgsks_list_omp(
            C.byref(ker), karr, C.c_int(ntask), C.c_int(k), _p(u), C.c_int(u.size),
            _p(a_off), _p(a_idx), _p(u_idx), _p(b_off), _p(b_idx), _p(w_idx),
            _p(XA), _p(XA2), _p(XB), _p(XB2), _p(w)))
    if impl == "reference":
        assert kers is None and np.array_equal(a_idx, u_idx) and np.array_equal(b_idx, w_idx)
        _lib("reference")
        _lib("shim").ref_omp_dgsks_list_flat(
            C.byref(ker), C.c_int(k), C.c_int(u.size), _p(u), C.c_int(ntask),
            _p(a_off), _p(a_idx), _p(b_off), _p(b_idx), _p(XA), _p(XA2), _p(XB), _p(XB2), _p(w))
        return 0
    raise ValueError(impl)


# ---------------------------------------------------------------------------
# Error metrics (normwise, conditioned max / rms relative).
def errors(u_test, u_ref, cond=None) -> dict:
    """Normwise ||du||/||u_ref|| (reference test/test_dgsks.c:43-79) and, when
    cond = sum_j |K_ij w_j| is given, max and rms of |du_i| / cond_i."""
    du = np.asarray(u_test, dtype=np.float64) - np.asarray(u_ref, dtype=np.float64)
    nrm = float(np.linalg.norm(u_ref))
    out = {"normwise": float(np.linalg.norm(du) / nrm) if nrm > 0 else float(np.linalg.norm(du))}
    if cond is not None:
        c = np.where(np.asarray(cond) > 0, cond, 1.0)
        r = np.abs(du) / c
        out["cond_max"] = float(r.max()) if r.size else 0.0
        out["cond_rms"] = float(np.sqrt(np.mean(r * r))) if r.size else 0.0
    return out
