"""Host-pointer calls gather their rows either with a kernel that reads the
caller's (pageable) host arrays, on devices that read host memory coherently,
or on the host into pinned buffers (GSKS_HOST_GATHER=cpu).  Both must give
the same bits, in both precisions, for the distance, inner-product and
variable-bandwidth kernels, with general-stride maps and several right-hand
sides; and a negative map entry must be refused before any kernel reads the
arrays.  The oracle checks the values."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(seed=5, N=3000, k=24, m=700, n=900):
    rng = np.random.default_rng(seed)
    X = rng.random((N, k))
    w = rng.standard_normal(N * 2)
    u0 = rng.standard_normal(N * 2)
    amap = rng.choice(N, m, replace=False).astype(np.int32)
    bmap = rng.choice(N, n, replace=False).astype(np.int32)
    umap = rng.permutation(N)[:m].astype(np.int32)
    wmap = rng.permutation(N)[:n].astype(np.int32)
    return X, w, u0, amap, bmap, umap, wmap


KERNELS = [(0, dict(scal=-2.0)), (2, {}), (1, dict(scal=0.1, cons=0.5, powe=3.0)), (3, {})]


@pytest.mark.parametrize("ktype,params", KERNELS, ids=["gaussian", "laplace", "polynomial", "varbw"])
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "split"])
def test_gather_paths_agree_bitwise(gpu, oracle_mod, monkeypatch, ktype, params, precision):
    from ks_gb300 import gsks
    O = oracle_mod
    X, w, u0, amap, bmap, umap, wmap = _case()
    X2 = O.norms(X)
    kp = dict(params)
    if ktype == 3:
        h = np.exp(np.random.default_rng(9).uniform(np.log(0.1), np.log(0.7), X.shape[0]))
        kp.update(hi=1.0 / h ** 2, hj=1.0 / h ** 2)
    wv, uv = w[: X.shape[0]], u0[: X.shape[0]]
    prev = gsks.get_precision()
    gsks.set_precision(precision)
    try:
        outs = {}
        for mode in ("device", "cpu"):
            if mode == "cpu":
                monkeypatch.setenv("GSKS_HOST_GATHER", "cpu")
            else:
                monkeypatch.delenv("GSKS_HOST_GATHER", raising=False)
            u = uv.copy()
            rc = gsks.dgsks_status(gsks.make_kernel(ktype, **kp), u, umap, X, X2, amap, X, X2, bmap, wv, wmap)
            assert rc == 0, gsks.error_string(rc)
            outs[mode] = u
            # two right-hand sides, interleaved
            u2 = u0.copy()
            rc = gsks.dgsks_rhs(gsks.make_kernel(ktype, **kp), 2, u2, umap, X, X2, amap, X, X2, bmap, w, wmap)
            assert rc == 0, gsks.error_string(rc)
            outs[mode + "_rhs"] = u2
    finally:
        gsks.set_precision(prev)
    assert np.array_equal(outs["device"], outs["cpu"])
    assert np.array_equal(outs["device_rhs"], outs["cpu_rhs"])
    ref = uv.copy()
    O.dgsks(O.make_kernel(ktype, **kp), ref, umap, X, X2, amap, X, X2, bmap, wv, wmap)
    tol = 1e-12 if precision == 0 else 1e-6
    assert np.linalg.norm(outs["device"] - ref) <= tol * np.linalg.norm(ref - uv)


def test_gather_mode_query_and_map_check(gpu, monkeypatch):
    from ks_gb300 import gsks
    monkeypatch.delenv("GSKS_HOST_GATHER", raising=False)
    on_device = gsks.host_gather_on_device()
    monkeypatch.setenv("GSKS_HOST_GATHER", "cpu")
    assert gsks.host_gather_on_device() is False
    monkeypatch.delenv("GSKS_HOST_GATHER", raising=False)
    assert gsks.host_gather_on_device() == on_device
    X, w, u0, amap, bmap, umap, wmap = _case(seed=6)
    X2 = np.einsum("ij,ij->i", X, X)
    for bad in ("amap", "bmap", "umap", "wmap"):
        maps = dict(amap=amap.copy(), bmap=bmap.copy(), umap=umap.copy(), wmap=wmap.copy())
        maps[bad][len(maps[bad]) // 2] = -3
        u = u0[: X.shape[0]].copy()
        rc = gsks.dgsks_status(gsks.make_kernel(0, scal=-1.0), u, maps["umap"], X, X2, maps["amap"], X, X2,
                               maps["bmap"], w[: X.shape[0]], maps["wmap"])
        assert rc == gsks.GSKS_ERR_MAP_RANGE, (bad, gsks.error_string(rc))
        assert np.array_equal(u, u0[: X.shape[0]])
