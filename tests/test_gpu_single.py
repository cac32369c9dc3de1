"""sgsks (FP32 arrays) against the oracle evaluated on the same FP32 values in
FP64.  The result is stored in FP32, so the gate is the split form's: 1e-6
normwise and conditioned, in both precisions of the evaluation.  u carries its
initial values, whose FP32 rounding is part of the result: the conditioned
metric divides by sum_j |K_ij w_j| + |u0_i|."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-6
KERNELS = [(0, dict(scal=-2.0)), (2, {}), (1, dict(scal=1.0 / 16, cons=1.0, powe=3.0))]


def _case(seed, N, k, m, n):
    rng = np.random.default_rng(seed)
    X = rng.random((N, k)).astype(np.float32)
    w = rng.standard_normal(N).astype(np.float32)
    u0 = rng.standard_normal(N).astype(np.float32)
    amap = rng.choice(N, m, replace=False).astype(np.int32)
    bmap = rng.choice(N, n, replace=False).astype(np.int32)
    umap = rng.permutation(N)[:m].astype(np.int32)
    wmap = rng.permutation(N)[:n].astype(np.int32)
    return X, w, u0, amap, bmap, umap, wmap


def _reference(O, ktype, params, X, w, u0, amap, bmap, umap, wmap):
    Xd, wd = X.astype(np.float64), w.astype(np.float64)
    X2 = O.norms(Xd)
    u_ref = u0.astype(np.float64)
    O.dgsks(O.make_kernel(ktype, **params), u_ref, umap, Xd, X2, amap, Xd, X2, bmap, wd, wmap)
    _, cond = O.rows(O.make_kernel(ktype, **params), np.arange(amap.size, dtype=np.int32), Xd, X2, amap, Xd, X2,
                     bmap, wd, wmap)
    return u_ref, cond


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("ktype,params", KERNELS)
def test_sgsks_host(gpu, oracle_mod, prec, ktype, params):
    from ks_gb300 import gsks
    O = oracle_mod
    X, w, u0, amap, bmap, umap, wmap = _case(70 + ktype, 5000, 16, 800, 1000)
    u_ref, cond = _reference(O, ktype, params, X, w, u0, amap, bmap, umap, wmap)
    u = u0.copy()
    prev = gsks.get_precision()
    gsks.set_precision(prec)
    try:
        rc = gsks.sgsks_status(gsks.make_kernel(ktype, **params), u, umap, X, None, amap, X, None, bmap, w, wmap)
    finally:
        gsks.set_precision(prev)
    assert rc == 0, gsks.error_string(rc)
    assert u.dtype == np.float32
    e = O.errors(u[umap].astype(np.float64), u_ref[umap], cond=cond + np.abs(u0[umap].astype(np.float64)))
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e
    untouched = np.setdiff1d(np.arange(5000), umap)
    assert np.array_equal(u[untouched], u0[untouched])


@pytest.mark.parametrize("prec", [0, 1])
def test_sgsks_device(gpu, oracle_mod, prec):
    from ks_gb300 import gsks
    torch = gpu
    O = oracle_mod
    X, w, u0, amap, bmap, umap, wmap = _case(80, 6000, 40, 1200, 1500)
    u_ref, cond = _reference(O, 0, dict(scal=-0.5), X, w, u0, amap, bmap, umap, wmap)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    u = t(u0)
    prev = gsks.get_precision()
    gsks.set_precision(prec)
    try:
        rc = gsks.sgsks_status(gsks.make_kernel(0, scal=-0.5), u, t(umap), t(X), None, t(amap), t(X), None,
                               t(bmap), t(w), t(wmap))
    finally:
        gsks.set_precision(prev)
    assert rc == 0, gsks.error_string(rc)
    got = u.cpu().numpy().astype(np.float64)
    e = O.errors(got[umap], u_ref[umap], cond=cond + np.abs(u0[umap].astype(np.float64)))
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e


def test_sgsks_negative_map_refused(gpu):
    from ks_gb300 import gsks
    X, w, u0, amap, bmap, umap, wmap = _case(81, 2000, 8, 300, 300)
    bmap[7] = -1
    u = u0.copy()
    rc = gsks.sgsks_status(gsks.make_kernel(0, scal=-0.5), u, umap, X, None, amap, X, None, bmap, w, wmap)
    assert rc == 5, gsks.error_string(rc)
    assert np.array_equal(u, u0)
