"""C-ABI surface of libgsks.so without a GPU: the library loads, exports
every function include/*.h declares, and its host-side argument checks return
the documented status codes before any device work."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT

HEADERS = [os.path.join(ROOT, "include", f) for f in sorted(os.listdir(os.path.join(ROOT, "include")))
           if f.endswith(".h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        src = re.sub(r"#[^\n]*", "", src)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_\s\*]*?)\b([a-z_][a-z0-9_]*)\s*\(([^;{]*?)\)\s*;", src):
            ret, name = m.group(1).strip(), m.group(2)
            if ret and not ret.startswith("typedef") and name not in ("if", "while", "sizeof"):
                names.add(name)
    return sorted(names)


def test_headers_declare_the_reference_surface():
    names = declared_functions()
    for ref_name in ("dgsks", "dgsks_ref", "ks_malloc_aligned", "dgsks_wrapper", "dgsks_ref_wrapper"):
        assert ref_name in names
    assert "dgsks_list" in names and "gsks_dgsks_device" in names


def test_library_exports_every_declared_symbol(gsks_lib):
    missing = [n for n in declared_functions() if not hasattr(gsks_lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_ks_t_layout():
    from ks_gb300.gsks import KsT
    # enum (4 bytes, padded to 8) + 3 doubles + 3 pointers = 56 bytes (reference include/ks.h:60-71)
    assert C.sizeof(KsT) == 56
    assert KsT.powe.offset == 8 and KsT.hi.offset == 32 and KsT.h.offset == 48


def _args(m=4, n=3, k=5, N=8):
    rng = np.random.default_rng(0)
    X = rng.random((N, k)); X2 = (X * X).sum(1)
    idx = np.arange(N, dtype=np.int32)
    return dict(u=np.zeros(N), umap=idx[:m].copy(), XA=X, XA2=X2, amap=idx[:m].copy(),
                XB=X, XB2=X2, bmap=idx[:n].copy(), w=np.ones(N), wmap=idx[:n].copy())


def _call(ker, a, k=None):
    from ks_gb300 import gsks
    return gsks.dgsks_status(ker, a["u"], a["umap"], a["XA"], a["XA2"], a["amap"], a["XB"], a["XB2"],
                             a["bmap"], a["w"], a["wmap"], k=k)


def test_status_codes_without_device(gsks_lib):
    from ks_gb300 import gsks
    a = _args()
    assert _call(gsks.make_kernel(11), a) == 2            # illegal type (reference exits, dgsks.c:465-467)
    assert gsks.last_error() == 2
    assert _call(gsks.make_kernel(gsks.KS_GAUSSIAN_VAR_BANDWIDTH), a) == 3   # no hi/hj
    assert _call(gsks.make_kernel(gsks.KS_LAPLACE), _args(k=2), k=2) == 4    # Laplace k < 3
    ker = gsks.make_kernel(gsks.KS_GAUSSIAN, scal=-0.5)
    assert gsks.load().dgsks_status(C.byref(ker), -1, 3, 5, *([None] * 10)) == 1
    assert np.all(a["u"] == 0.0)
    assert "laplace" in gsks.error_string(4)


def test_early_return_precedes_type_checks(gsks_lib):
    """m, n or k == 0 returns before the kernel switch (frame/dgsks.c:394-397)."""
    from ks_gb300 import gsks
    a = _args(m=0)
    ker = gsks.make_kernel(gsks.KS_LAPLACE)
    assert _call(ker, a) == 0
    assert ker.powe == 1.0 and ker.scal == 0.0       # untouched
    assert _call(gsks.make_kernel(11), _args(n=0)) == 0


def test_precision_switch(gsks_lib):
    from ks_gb300 import gsks
    with pytest.raises(gsks.GsksError):
        gsks.set_precision(7)
    gsks.set_precision(gsks.GSKS_FP64)
    assert gsks.get_precision() == gsks.GSKS_FP64


def test_ks_malloc_aligned(gsks_lib):
    from ks_gb300 import gsks
    lib = gsks.load()
    p = lib.ks_malloc_aligned(100, 7, 8)
    assert p and p % 64 == 0
    C.CDLL(None).free(C.c_void_p(p))


def test_python_binding_checks(gsks_lib):
    from ks_gb300 import gsks
    a = _args()
    with pytest.raises(ValueError):
        gsks.dgsks(5, a["u"], a["umap"], a["XA"], a["XA2"], a["amap"], a["XB"], a["XB2"], a["bmap"],
                   a["w"], a["wmap"], type="Nope")
