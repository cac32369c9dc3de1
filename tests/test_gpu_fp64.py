"""Plain FP64 form on the GPU against the oracle and the reference's golden
vectors: the ks.h host-pointer path, the device-pointer path, the unfused
dgsks_ref, and determinism.  Tolerance 1e-12 (normwise, and conditioned
max-relative |du_i| / sum_j |K_ij w_j|)."""
import numpy as np
import pytest

from conftest import golden_manifest, load_golden

pytestmark = pytest.mark.gpu

MANIFEST = golden_manifest()
SINGLE = sorted(k for k, v in MANIFEST.items() if "ntask" not in v)
TOL = 1e-12


def _kernel(mod, meta, hi=None):
    extra = {"hi": hi, "hj": hi} if hi is not None else {}
    return mod.make_kernel(meta["type"], **meta["params"], **extra)


def _cond(O, meta, g):
    hi = g["hi"] if g["hi"].size > 1 else None
    rows = np.arange(meta["m"], dtype=np.int32)
    s, a = O.rows(_kernel(O, meta, hi), rows, g["X"], g["X2"], g["amap"], g["X"], g["X2"], g["bmap"],
                  g["w"], g["wmap"])
    return a


def _check(O, meta, g, u, tol=TOL):
    umap = g["umap"]
    err = O.errors(u[umap], g["u_ref"][umap], cond=_cond(O, meta, g) + np.abs(g["u0"][umap]))
    assert err["normwise"] <= tol, err
    assert err["cond_max"] <= tol, err
    touched = np.zeros(u.size, bool); touched[umap] = True
    assert np.array_equal(u[~touched], g["u0"][~touched])


@pytest.mark.parametrize("name", SINGLE)
def test_host_path_matches_reference(gpu, oracle_mod, name):
    from ks_gb300 import gsks
    meta, g = MANIFEST[name], load_golden(name)
    hi = g["hi"] if g["hi"].size > 1 else None
    ker = _kernel(gsks, meta, hi)
    u = g["u0"].copy()
    gsks.set_precision(gsks.GSKS_FP64)
    rc = gsks.dgsks_status(ker, u, g["umap"], g["X"], g["X2"], g["amap"], g["X"], g["X2"], g["bmap"], g["w"], g["wmap"])
    assert rc == 0, gsks.error_string(rc)
    _check(oracle_mod, meta, g, u)
    assert ker.powe == float(g["powe_after"]) and ker.scal == float(g["scal_after"])


@pytest.mark.parametrize("name", SINGLE)
def test_device_path_matches_reference(gpu, oracle_mod, name):
    from ks_gb300 import gsks
    torch = gpu
    meta, g = MANIFEST[name], load_golden(name)
    d = {k: torch.from_numpy(v).cuda() for k, v in g.items() if k in ("X", "X2", "w", "u0", "hi", "amap", "bmap", "umap", "wmap")}
    hi = d["hi"] if g["hi"].size > 1 else None
    ker = _kernel(gsks, meta, hi)
    u = d["u0"].clone()
    N, k = g["X"].shape
    gsks.dgsks_device(ker, meta["m"], meta["n"], k, u, d["umap"], d["X"], d["X2"], d["amap"], d["X"], d["X2"],
                      d["bmap"], d["w"], d["wmap"], stream=torch.cuda.current_stream(), nxa=N, nxb=N)
    assert gsks.last_launch_count() >= 2
    torch.cuda.synchronize()
    _check(oracle_mod, meta, g, u.cpu().numpy())


@pytest.mark.parametrize("name", ["gauss_general", "laplace_k37", "poly3_general", "tanh_general",
                                  "varbw_general", "quartic_general", "gauss_k300", "gauss_tails"])
def test_unfused_dgsks_ref_matches_reference(gpu, oracle_mod, name):
    from ks_gb300 import gsks
    meta, g = MANIFEST[name], load_golden(name)
    hi = g["hi"] if g["hi"].size > 1 else None
    u = g["u0"].copy()
    rc = gsks.dgsks_ref_call(_kernel(gsks, meta, hi), u, g["umap"], g["X"], g["X2"], g["amap"], g["X"], g["X2"],
                             g["bmap"], g["w"], g["wmap"])
    assert rc == 0
    _check(oracle_mod, meta, g, u)


def _random_case(seed, N, k, m, n):
    rng = np.random.default_rng(seed)
    X = rng.random((N, k))
    X2 = (X * X).sum(1)
    w = rng.standard_normal(N)
    amap = rng.choice(N, m, replace=False).astype(np.int32)
    bmap = rng.choice(N, n, replace=False).astype(np.int32)
    umap = rng.permutation(N)[:m].astype(np.int32)
    wmap = rng.permutation(N)[:n].astype(np.int32)
    return X, X2, w, amap, bmap, umap, wmap


@pytest.mark.parametrize("ktype,params", [(0, dict(scal=-2.0)), (2, {}), (1, dict(scal=1 / 64, cons=1.0, powe=3.0))])
def test_general_stride_config2_shape(gpu, oracle_mod, ktype, params):
    """The general-stride configuration's shape (k=64, random subsets of a larger
    pool, permuted u/w maps) at a size the oracle evaluates in seconds."""
    from ks_gb300 import gsks
    O = oracle_mod
    X, X2, w, amap, bmap, umap, wmap = _random_case(7, 12000, 64, 3000, 2500)
    # norms summed in the same order as the oracle's inner products, so that
    # coincident points cancel exactly there (Laplace is singular at d2 = 0)
    X2 = O.norms(X)
    u_ref = np.zeros(12000)
    O.dgsks(O.make_kernel(ktype, **params), u_ref, umap, X, X2, amap, X, X2, bmap, w, wmap)
    _, cond = O.rows(O.make_kernel(ktype, **params), np.arange(3000, dtype=np.int32), X, X2, amap, X, X2, bmap, w, wmap)
    u = np.zeros(12000)
    assert gsks.dgsks_status(gsks.make_kernel(ktype, **params), u, umap, X, X2, amap, X, X2, bmap, w, wmap) == 0
    err = O.errors(u[umap], u_ref[umap], cond=cond)
    assert err["normwise"] <= TOL and err["cond_max"] <= TOL, err


def test_deterministic(gpu):
    from ks_gb300 import gsks
    X, X2, w, amap, bmap, umap, wmap = _random_case(8, 20000, 32, 9000, 11000)
    outs = []
    for _ in range(2):
        u = np.zeros(20000)
        assert gsks.dgsks_status(gsks.make_kernel(0, scal=-1.0), u, umap, X, X2, amap, X, X2, bmap, w, wmap) == 0
        outs.append(u)
    assert np.array_equal(outs[0], outs[1])


def test_accumulates_into_u(gpu):
    """u is in/out: a second call adds the same sums again (frame/dgsks_ref.c:434-435)."""
    from ks_gb300 import gsks
    X, X2, w, amap, bmap, umap, wmap = _random_case(9, 2000, 8, 500, 400)
    u1 = np.zeros(2000)
    ker = gsks.make_kernel(0, scal=-0.5)
    gsks.dgsks_status(ker, u1, umap, X, X2, amap, X, X2, bmap, w, wmap)
    u2 = u1.copy()
    gsks.dgsks_status(ker, u2, umap, X, X2, amap, X, X2, bmap, w, wmap)
    assert np.allclose(u2[umap], 2 * u1[umap], rtol=1e-13, atol=0)


def test_device_map_range_flag(gpu):
    """An out-of-range map index on the device path is clamped and flagged, not read."""
    from ks_gb300 import gsks
    torch = gpu
    X, X2, w, amap, bmap, umap, wmap = _random_case(10, 1000, 8, 100, 100)
    amap[5] = 5000
    t = lambda a: torch.from_numpy(a).cuda()
    u = torch.zeros(1000, dtype=torch.float64, device="cuda")
    gsks.dgsks_device(gsks.make_kernel(0, scal=-0.5), 100, 100, 8, u, t(umap), t(X), t(X2), t(amap), t(X),
                      t(X2), t(bmap), t(w), t(wmap), nxa=1000, nxb=1000)
    torch.cuda.synchronize()
    assert gsks.device_errors() & 1
    assert gsks.device_errors() == 0


@pytest.mark.parametrize("which", ["amap", "umap", "bmap", "wmap"])
def test_host_map_negative_index_refused(gpu, which):
    """Host arrays: a negative index in any map returns GSKS_ERR_MAP_RANGE and
    leaves u unchanged (the maps are checked while the rows are gathered, large
    enough here for several gather chunks)."""
    from ks_gb300 import gsks
    X, X2, w, amap, bmap, umap, wmap = _random_case(12, 40000, 64, 20000, 20000)
    maps = dict(amap=amap, umap=umap, bmap=bmap, wmap=wmap)
    maps[which][17000] = -3
    u = np.full(40000, 2.5)
    for prec in (gsks.GSKS_FP64, gsks.GSKS_SPLIT_BF16X3):
        prev = gsks.get_precision()
        gsks.set_precision(prec)
        try:
            rc = gsks.dgsks_status(gsks.make_kernel(0, scal=-0.5), u, maps["umap"], X, X2, maps["amap"], X, X2,
                                   maps["bmap"], w, maps["wmap"])
        finally:
            gsks.set_precision(prev)
        assert rc == 5, gsks.error_string(rc)
        assert np.all(u == 2.5)


def test_c1_configuration_as_stated(gpu, oracle_mod):
    """The CPU-runnable configuration exactly: m = n = 2048 targets and sources,
    k = 16, points U[0,1]^16, norms in FP64, w ~ N(0,1), identity maps,
    Gaussian h = 1 (scal = -1/(2h^2) = -0.5), seed-generated.  Checked as the
    reference's own test does (test/test_dgsks.c:41,43-79): the normwise error
    against dgsks_ref within 1e-13; the split form within its 1e-6 gate."""
    from ks_gb300 import gsks
    O = oracle_mod
    rng = np.random.default_rng(2048)
    N, k = 2048, 16
    X = rng.random((N, k))
    X2 = O.norms(X)
    w = rng.standard_normal(N)
    ident = np.arange(N, dtype=np.int32)
    u_ref = np.zeros(N)
    O.dgsks(O.make_kernel(0, scal=-0.5), u_ref, ident, X, X2, ident, X, X2, ident, w, ident)
    _, cond = O.rows(O.make_kernel(0, scal=-0.5), ident, X, X2, ident, X, X2, ident, w, ident)
    prev = gsks.get_precision()
    try:
        for prec, tol in ((gsks.GSKS_FP64, 1e-13), (gsks.GSKS_SPLIT_BF16X3, 1e-6)):
            gsks.set_precision(prec)
            u = np.zeros(N)
            rc = gsks.dgsks_status(gsks.make_kernel(0, scal=-0.5), u, ident, X, X2, ident, X, X2, ident, w, ident)
            assert rc == 0, gsks.error_string(rc)
            e = O.errors(u, u_ref, cond=cond)
            assert e["normwise"] <= tol and e["cond_max"] <= tol, (prec, e)
    finally:
        gsks.set_precision(prev)
