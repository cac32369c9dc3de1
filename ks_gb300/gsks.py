"""Python host interface of the GB300 GSKS library (ctypes over libgsks.so).

Mirrors the reference's Python binding ``python/gsks.py`` (``dgsks`` at
python/gsks.py:112-199, ``dgsks_ref`` at :18-105): same argument order and
meaning, keyword options ``type``, ``scal``, ``cons``, ``powe`` and ``h``.
Differences from the reference binding: Python 3, ``cons`` is forwarded
(the reference writes it into ``scal``, python/gsks.py:53-54,66-67,74), nothing
is printed, and a failed call raises ``GsksError`` with the library status.

Lower-level entry points expose the rest of the C ABI: ``dgsks_device`` (device
pointers, e.g. torch tensors, on a CUDA stream), ``dgsks_list`` (flat CSR
batched call), ``set_precision``.  There is no CPU fallback: if libgsks.so is
missing the import-time ``load()`` raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("GSKS_LIB", os.path.join(_PKG, "lib", "libgsks.so"))

KS_GAUSSIAN, KS_POLYNOMIAL, KS_LAPLACE, KS_GAUSSIAN_VAR_BANDWIDTH = 0, 1, 2, 3
KS_TANH, KS_QUARTIC, KS_MULTIQUADRATIC, KS_EPANECHNIKOV = 4, 5, 6, 7
GSKS_FP64, GSKS_SPLIT_BF16X3 = 0, 1
GSKS_ERR_MAP_RANGE, GSKS_ERR_TIMEOUT = 5, 12

# option "type" strings of python/gsks.py:47-79
TYPE_NAMES = {
    "Gaussian": KS_GAUSSIAN, "Polynomial": KS_POLYNOMIAL, "Laplace": KS_LAPLACE,
    "Variable_Bandwidth": KS_GAUSSIAN_VAR_BANDWIDTH, "Tanh": KS_TANH,
    "Quartic": KS_QUARTIC, "Multiquadratic": KS_MULTIQUADRATIC,
    "Epanechnikov": KS_EPANECHNIKOV,
}


class GsksError(RuntimeError):
    def __init__(self, code: int, where: str):
        self.code = code
        super().__init__(f"{where}: {error_string(code)} (status {code})")


class KsT(C.Structure):
    """ks_t (include/ks.h): type, powe, scal, cons, hi, hj, h."""
    _fields_ = [("type", C.c_int), ("powe", C.c_double), ("scal", C.c_double),
                ("cons", C.c_double), ("hi", C.c_void_p), ("hj", C.c_void_p),
                ("h", C.c_void_p)]


_lib = None


def load():
    """Load libgsks.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libgsks.so not found at {LIB_PATH}; run ks_gb300.build.build()")
    lib = C.CDLL(LIB_PATH)
    vp, ip, dp = C.c_void_p, C.c_int, C.c_double
    lib.dgsks_status.restype = C.c_int
    lib.gsks_dgsks_device.restype = C.c_int
    lib.gsks_dgsks_device.argtypes = [C.POINTER(KsT), ip, ip, ip, vp, vp, vp, vp, vp, ip,
                                      vp, vp, vp, ip, vp, vp, ip, vp]
    lib.gsks_dgsks_device_rhs.restype = C.c_int
    lib.gsks_dgsks_device_rhs.argtypes = [C.POINTER(KsT), ip, ip, ip, ip, vp, vp, vp, vp, vp, ip,
                                          vp, vp, vp, ip, vp, vp, ip, vp]
    lib.dgsks_rhs.restype = C.c_int
    lib.sgsks_status.restype = C.c_int
    lib.gsks_norms_device.restype = C.c_int
    lib.gsks_norms_device.argtypes = [ip, ip, vp, vp, vp]
    lib.gsks_error_string.restype = C.c_char_p
    lib.gsks_last_error.restype = C.c_int
    lib.gsks_set_precision.restype = C.c_int
    lib.gsks_get_precision.restype = C.c_int
    lib.gsks_last_launch_count.restype = C.c_int
    lib.gsks_device_errors.restype = C.c_int
    lib.ks_malloc_aligned.restype = vp
    lib.ks_malloc_aligned.argtypes = [ip, ip, ip]
    if hasattr(lib, "dgsks_list"):
        lib.dgsks_list.restype = C.c_int
    lib.gsks_list_plan_create.restype = C.c_int
    lib.gsks_list_plan_create.argtypes = [C.POINTER(vp), C.POINTER(KsT), vp, ip, ip, ip, vp, vp, vp, vp, vp, vp,
                                          ip, ip, ip, ip, ip]
    lib.gsks_list_plan_execute.restype = C.c_int
    lib.gsks_list_plan_execute.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp]
    lib.gsks_list_plan_errors.restype = C.c_int
    lib.gsks_list_plan_errors.argtypes = [vp]
    lib.gsks_list_plan_destroy.restype = C.c_int
    lib.gsks_list_plan_destroy.argtypes = [vp]
    lib.gsks_split_stats.restype = C.c_int
    lib.gsks_split_stats.argtypes = [C.POINTER(C.c_longlong), C.POINTER(C.c_int)]
    lib.gsks_split_test_wait.restype = C.c_int
    lib.gsks_split_test_wait.argtypes = [C.c_longlong, C.c_int]
    _lib = lib
    return lib


def error_string(code: int) -> str:
    return load().gsks_error_string(C.c_int(code)).decode()


def last_error() -> int:
    return int(load().gsks_last_error())


def last_launch_count() -> int:
    return int(load().gsks_last_launch_count())


def device_errors() -> int:
    """Device-side error flags of this thread's context (read and cleared)."""
    return int(load().gsks_device_errors())


def split_stats() -> dict:
    """Rechecked pairs and rescued rows of this thread's last single
    split-precision call (waits for the device)."""
    r, q = C.c_longlong(), C.c_int()
    rc = load().gsks_split_stats(C.byref(r), C.byref(q))
    if rc:
        raise GsksError(rc, "gsks_split_stats")
    return {"rechecked_pairs": int(r.value), "rescued_rows": int(q.value)}


def host_gather_on_device() -> bool:
    """Whether host-pointer calls gather their rows with a kernel reading the
    caller's arrays (devices that read pageable host memory; not with
    GSKS_HOST_GATHER=cpu) rather than on the host (gsks.h)."""
    return load().gsks_host_gather_on_device() == 1


def split_test_wait(wait_cycles: int = 0, stall: bool = False) -> None:
    """Test hook: bounded-wait limit (clock cycles, 0 = default) and producer
    stall of this thread's later split-precision calls (gsks.h)."""
    load().gsks_split_test_wait(C.c_longlong(int(wait_cycles)), C.c_int(1 if stall else 0))


def set_precision(p: int) -> None:
    rc = load().gsks_set_precision(C.c_int(p))
    if rc:
        raise GsksError(rc, "gsks_set_precision")


def get_precision() -> int:
    return int(load().gsks_get_precision())


def make_kernel(ktype, scal=0.0, cons=0.0, powe=1.0, hi=None, hj=None) -> KsT:
    """Descriptor; hi/hj may be numpy arrays, torch tensors or raw addresses."""
    ker = KsT()
    ker.type = int(ktype)
    ker.scal, ker.cons, ker.powe = float(scal), float(cons), float(powe)
    ker.hi = _addr(hi) if hi is not None else None
    ker.hj = _addr(hj) if hj is not None else None
    ker.h = None
    return ker


def _addr(a):
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if hasattr(a, "data_ptr"):       # torch.Tensor
        return a.data_ptr()
    return a.ctypes.data            # numpy


def _vp(a):
    return C.c_void_p(_addr(a))


def _host_check(dtype, *arrs):
    for a in arrs:
        if a is None:
            continue
        if not isinstance(a, np.ndarray) or not a.flags["C_CONTIGUOUS"]:
            raise TypeError("host arrays must be C-contiguous numpy arrays")


def dgsks_status(ker: KsT, u, umap, XA, XA2, amap, XB, XB2, bmap, w, wmap, k=None) -> int:
    """Raw ks.h dgsks() call with a status return; arrays may be host or device."""
    m = int(amap.numel() if hasattr(amap, "numel") else amap.size)
    n = int(bmap.numel() if hasattr(bmap, "numel") else bmap.size)
    if k is None:
        k = int(XA.shape[1])
    return int(load().dgsks_status(
        C.byref(ker), C.c_int(m), C.c_int(n), C.c_int(k), _vp(u), _vp(umap), _vp(XA), _vp(XA2),
        _vp(amap), _vp(XB), _vp(XB2), _vp(bmap), _vp(w), _vp(wmap)))


def sgsks_status(ker: KsT, u, umap, XA, XA2, amap, XB, XB2, bmap, w, wmap, k=None) -> int:
    """Single precision (gsks.h sgsks_status): FP32 u, XA, XB, w (host or device);
    XA2/XB2 may be None (recomputed in FP64).  Returns the status."""
    m = int(amap.numel() if hasattr(amap, "numel") else amap.size)
    n = int(bmap.numel() if hasattr(bmap, "numel") else bmap.size)
    if k is None:
        k = int(XA.shape[1])
    return int(load().sgsks_status(
        C.byref(ker), C.c_int(m), C.c_int(n), C.c_int(k), _vp(u), _vp(umap), _vp(XA), _vp(XA2),
        _vp(amap), _vp(XB), _vp(XB2), _vp(bmap), _vp(w), _vp(wmap)))


def dgsks_ref_call(ker: KsT, u, umap, XA, XA2, amap, XB, XB2, bmap, w, wmap, k=None) -> int:
    """ks.h dgsks_ref() (unfused GPU evaluation); returns the status."""
    m = int(amap.numel() if hasattr(amap, "numel") else amap.size)
    n = int(bmap.numel() if hasattr(bmap, "numel") else bmap.size)
    if k is None:
        k = int(XA.shape[1])
    lib = load()
    lib.dgsks_ref(C.byref(ker), C.c_int(m), C.c_int(n), C.c_int(k), _vp(u), _vp(umap), _vp(XA),
                  _vp(XA2), _vp(amap), _vp(XB), _vp(XB2), _vp(bmap), _vp(w), _vp(wmap))
    return last_error()


def dgsks_device(ker: KsT, m, n, k, u, umap, XA, XA2, amap, XB, XB2, bmap, w, wmap,
                 precision=GSKS_FP64, stream=None, nxa=-1, nxb=-1) -> None:
    """Enqueue a device-resident evaluation (all pointers on the device)."""
    s = stream if isinstance(stream, int) or stream is None else stream.cuda_stream
    rc = load().gsks_dgsks_device(
        C.byref(ker), m, n, k, _addr(u), _addr(umap), _addr(XA), _addr(XA2), _addr(amap), nxa,
        _addr(XB), _addr(XB2), _addr(bmap), nxb, _addr(w), _addr(wmap), int(precision), s)
    if rc:
        raise GsksError(rc, "gsks_dgsks_device")


def dgsks_device_rhs(ker: KsT, m, n, k, nrhs, u, umap, XA, XA2, amap, XB, XB2, bmap, w, wmap,
                     precision=GSKS_FP64, stream=None, nxa=-1, nxb=-1) -> None:
    """dgsks_device with nrhs interleaved right-hand sides:
    u[umap[i]*nrhs + r] += sum_j K_ij w[wmap[j]*nrhs + r]."""
    s = stream if isinstance(stream, int) or stream is None else stream.cuda_stream
    rc = load().gsks_dgsks_device_rhs(
        C.byref(ker), m, n, k, int(nrhs), _addr(u), _addr(umap), _addr(XA), _addr(XA2), _addr(amap), nxa,
        _addr(XB), _addr(XB2), _addr(bmap), nxb, _addr(w), _addr(wmap), int(precision), s)
    if rc:
        raise GsksError(rc, "gsks_dgsks_device_rhs")


def dgsks_rhs(ker: KsT, nrhs, u, umap, XA, XA2, amap, XB, XB2, bmap, w, wmap, k=None) -> int:
    """Synchronous multi-rhs call (gsks.h dgsks_rhs); host or device arrays; the status."""
    m = int(amap.numel() if hasattr(amap, "numel") else amap.size)
    n = int(bmap.numel() if hasattr(bmap, "numel") else bmap.size)
    if k is None:
        k = int(XA.shape[1])
    return int(load().dgsks_rhs(
        C.byref(ker), C.c_int(m), C.c_int(n), C.c_int(k), C.c_int(int(nrhs)), _vp(u), _vp(umap), _vp(XA),
        _vp(XA2), _vp(amap), _vp(XB), _vp(XB2), _vp(bmap), _vp(w), _vp(wmap)))


def norms_device(X, X2, stream=None) -> None:
    s = stream if isinstance(stream, int) or stream is None else stream.cuda_stream
    N, k = int(X.shape[0]), int(X.shape[1])
    rc = load().gsks_norms_device(N, k, _addr(X), _addr(X2), s)
    if rc:
        raise GsksError(rc, "gsks_norms_device")


def dgsks_list(ker: KsT, u, a_off, a_idx, b_off, b_idx, XA, XA2, XB, XB2, w,
               u_idx=None, w_idx=None, kers=None) -> None:
    """Flat batched call (gsks.h dgsks_list); arrays host (numpy) or device."""
    lib = load()
    ntask = int((a_off.numel() if hasattr(a_off, "numel") else a_off.size) - 1)
    k = int(XA.shape[1])
    karr = (KsT * ntask)(*kers) if kers is not None else None
    nu = int(u.numel() if hasattr(u, "numel") else u.size)
    nw = int(w.numel() if hasattr(w, "numel") else w.size)
    rc = lib.dgsks_list(C.byref(ker), karr, C.c_int(ntask), C.c_int(k), _vp(u), C.c_int(nu),
                        _vp(a_off), _vp(a_idx), _vp(u_idx), _vp(b_off), _vp(b_idx), _vp(w_idx),
                        _vp(XA), _vp(XA2), C.c_int(int(XA.shape[0])),
                        _vp(XB), _vp(XB2), C.c_int(int(XB.shape[0])), _vp(w), C.c_int(nw))
    if rc:
        raise GsksError(rc, "dgsks_list")


class ListPlan:
    """A planned dgsks_list (gsks.h gsks_list_plan_*): the lists, kernels and
    precision are fixed at construction; execute() evaluates for device
    tensors u, XA, XB, w (norms optional) and replays a CUDA graph when called
    again with the same tensors and stream.  Device lists must outlive the plan."""

    def __init__(self, ker: KsT, a_off, a_idx, b_off, b_idx, k: int, nu: int, nxa: int, nxb: int, nw: int,
                 u_idx=None, w_idx=None, kers=None, precision=GSKS_FP64, same_pool=False):
        lib = load()
        ntask = int((a_off.numel() if hasattr(a_off, "numel") else a_off.size) - 1)
        self._kers = (KsT * ntask)(*kers) if kers is not None else None
        self._keep = (ker, a_off, a_idx, b_off, b_idx, u_idx, w_idx, kers)
        h = C.c_void_p()
        rc = lib.gsks_list_plan_create(C.byref(h), C.byref(ker), C.cast(self._kers, C.c_void_p) if self._kers else None,
                                       ntask, int(k), int(nu), _vp(a_off), _vp(a_idx), _vp(u_idx), _vp(b_off),
                                       _vp(b_idx), _vp(w_idx), int(nxa), int(nxb), int(nw), int(precision),
                                       1 if same_pool else 0)
        if rc:
            raise GsksError(rc, "gsks_list_plan_create")
        self._h = h

    def execute(self, u, XA, XA2, XB, XB2, w, stream=None) -> None:
        s = None if stream is None else C.c_void_p(stream.cuda_stream)
        rc = load().gsks_list_plan_execute(self._h, _vp(u), _vp(XA), _vp(XA2), _vp(XB), _vp(XB2), _vp(w), s)
        if rc:
            raise GsksError(rc, "gsks_list_plan_execute")

    def errors(self) -> int:
        return int(load().gsks_list_plan_errors(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            load().gsks_list_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Reference-style interface (python/gsks.py).
def _options_kernel(options):
    t = options.get("type")
    if t not in TYPE_NAMES:
        raise ValueError(f"kernel option {t!r} is not supported")
    kt = TYPE_NAMES[t]
    scal = float(options.get("scal", 1.0) or 0.0)
    cons = float(options.get("cons", 0.0) or 0.0)
    powe = float(options.get("powe", 1.0) or 0.0)
    h = options.get("h")
    if kt == KS_GAUSSIAN_VAR_BANDWIDTH and h is None:
        raise ValueError("Variable_Bandwidth needs the h vector")
    return make_kernel(kt, scal=scal, cons=cons, powe=powe, hi=h, hj=h), h


def _check_args(d, u, mu, XA, XA2, alpha, XB, XB2, beta, w, omega):
    # range and type checks of python/gsks.py:19-37
    assert XA.shape[1] == XB.shape[1] == d
    assert XA.dtype == np.double and XB.dtype == np.double
    assert XA2.dtype == np.double and XB2.dtype == np.double
    assert XA2.size == XA.shape[0] and XB2.size == XB.shape[0]
    for a in (alpha, beta, mu, omega):
        assert a.dtype == np.int32
    _host_check(None, u, mu, XA, XA2, alpha, XB, XB2, beta, w, omega)


def dgsks(d, u, mu, XA, XA2, alpha, XB, XB2, beta, w, omega, **options):
    """u[mu[i]] += sum_j K(XA[alpha[i]], XB[beta[j]]) w[omega[j]] on the GPU."""
    _check_args(d, u, mu, XA, XA2, alpha, XB, XB2, beta, w, omega)
    ker, _h = _options_kernel(options)
    rc = dgsks_status(ker, u, mu, XA, XA2, alpha, XB, XB2, beta, w, omega, k=d)
    if rc:
        raise GsksError(rc, "dgsks")


def dgsks_ref(d, u, mu, XA, XA2, alpha, XB, XB2, beta, w, omega, **options):
    """Unfused GEMM + kernel + GEMV evaluation (GPU), same contract as dgsks."""
    _check_args(d, u, mu, XA, XA2, alpha, XB, XB2, beta, w, omega)
    ker, _h = _options_kernel(options)
    rc = dgsks_ref_call(ker, u, mu, XA, XA2, alpha, XB, XB2, beta, w, omega, k=d)
    if rc:
        raise GsksError(rc, "dgsks_ref")
