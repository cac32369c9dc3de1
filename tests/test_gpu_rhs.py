"""Several right-hand sides (dgsks_rhs, gsks_dgsks_device_rhs) against the
oracle run once per right-hand side: u and w hold nrhs interleaved columns,
u[umap[i]*nrhs + r] += sum_j K_ij w[wmap[j]*nrhs + r].

Gates: FP64 form 1e-12 (normwise and conditioned), split form 1e-6."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64, SPLIT = 0, 1
TOL = {FP64: 1e-12, SPLIT: 1e-6}
KERNELS = [(0, dict(scal=-2.0)), (2, {}), (1, dict(scal=1.0 / 16, cons=1.0, powe=3.0))]


def _case(seed, N, k, m, n, nrhs):
    rng = np.random.default_rng(seed)
    X = rng.random((N, k))
    w = rng.standard_normal(N * nrhs)
    amap = rng.choice(N, m, replace=False).astype(np.int32)
    bmap = rng.choice(N, n, replace=False).astype(np.int32)
    umap = rng.permutation(N)[:m].astype(np.int32)
    wmap = rng.permutation(N)[:n].astype(np.int32)
    u0 = rng.standard_normal(N * nrhs)
    return X, w, amap, bmap, umap, wmap, u0


def _reference(O, ktype, params, X, X2, w, amap, bmap, umap, wmap, u0, nrhs):
    u_ref = u0.copy()
    conds = []
    for r in range(nrhs):
        ur, wr = umap * nrhs + r, wmap * nrhs + r
        O.dgsks(O.make_kernel(ktype, **params), u_ref, ur.astype(np.int32), X, X2, amap, X, X2, bmap, w,
                wr.astype(np.int32))
        _, c = O.rows(O.make_kernel(ktype, **params), np.arange(amap.size, dtype=np.int32), X, X2, amap, X, X2,
                      bmap, w, wr.astype(np.int32))
        conds.append(c)
    return u_ref, np.stack(conds, axis=1)          # [m, nrhs]


def _check(O, got, u_ref, umap, cond, nrhs, tol):
    idx = (umap[:, None] * nrhs + np.arange(nrhs)[None, :]).ravel()
    e = O.errors(got[idx], u_ref[idx], cond=cond.ravel())
    assert e["normwise"] <= tol and e["cond_max"] <= tol, e


@pytest.mark.parametrize("prec", [FP64, SPLIT])
@pytest.mark.parametrize("ktype,params", KERNELS)
def test_rhs_host_arrays(gpu, oracle_mod, prec, ktype, params):
    from ks_gb300 import gsks
    O = oracle_mod
    nrhs = 3
    X, w, amap, bmap, umap, wmap, u0 = _case(40 + ktype, 5000, 16, 700, 900, nrhs)
    X2 = O.norms(X)
    u_ref, cond = _reference(O, ktype, params, X, X2, w, amap, bmap, umap, wmap, u0, nrhs)
    got = u0.copy()
    prev = gsks.get_precision()
    gsks.set_precision(prec)
    try:
        rc = gsks.dgsks_rhs(gsks.make_kernel(ktype, **params), nrhs, got, umap, X, X2, amap, X, X2, bmap, w, wmap)
    finally:
        gsks.set_precision(prev)
    assert rc == 0, gsks.error_string(rc)
    _check(O, got, u_ref, umap, cond, nrhs, TOL[prec])
    # entries no target names keep their values
    untouched = np.setdiff1d(np.arange(5000), umap)
    idx = (untouched[:, None] * nrhs + np.arange(nrhs)[None, :]).ravel()
    assert np.array_equal(got[idx], u0[idx])


@pytest.mark.parametrize("prec", [FP64, SPLIT])
def test_rhs_device_arrays(gpu, oracle_mod, prec):
    from ks_gb300 import gsks
    torch = gpu
    O = oracle_mod
    nrhs, ktype, params = 4, 0, dict(scal=-0.5)
    N, k, m, n = 6000, 24, 1100, 1300
    X, w, amap, bmap, umap, wmap, u0 = _case(50, N, k, m, n, nrhs)
    X2 = O.norms(X)
    u_ref, cond = _reference(O, ktype, params, X, X2, w, amap, bmap, umap, wmap, u0, nrhs)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    u = t(u0)
    gsks.dgsks_device_rhs(gsks.make_kernel(ktype, **params), m, n, k, nrhs, u, t(umap), t(X), t(X2), t(amap), t(X),
                          t(X2), t(bmap), t(w), t(wmap), precision=prec, stream=torch.cuda.current_stream(),
                          nxa=N, nxb=N)
    torch.cuda.synchronize()
    assert gsks.device_errors() == 0
    _check(O, u.cpu().numpy(), u_ref, umap, cond, nrhs, TOL[prec])


def test_rhs_one_equals_dgsks(gpu):
    """nrhs = 1 is dgsks itself, bit for bit."""
    from ks_gb300 import gsks
    X, w, amap, bmap, umap, wmap, u0 = _case(60, 3000, 8, 400, 500, 1)
    X2 = (X * X).sum(1)
    ker = gsks.make_kernel(0, scal=-1.0)
    a, b = u0.copy(), u0.copy()
    assert gsks.dgsks_status(ker, a, umap, X, X2, amap, X, X2, bmap, w, wmap) == 0
    assert gsks.dgsks_rhs(ker, 1, b, umap, X, X2, amap, X, X2, bmap, w, wmap) == 0
    assert np.array_equal(a, b)


def test_rhs_bad_count(gpu):
    from ks_gb300 import gsks
    X, w, amap, bmap, umap, wmap, u0 = _case(61, 1000, 8, 100, 100, 1)
    X2 = (X * X).sum(1)
    rc = gsks.dgsks_rhs(gsks.make_kernel(0, scal=-1.0), 0, u0, umap, X, X2, amap, X, X2, bmap, w, wmap)
    assert rc == 1, gsks.error_string(rc)
