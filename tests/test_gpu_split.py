"""Split-precision tensor-core form (tcgen05) against the FP64 oracle.

Tolerance 1e-6 on the normwise and the conditioned max-relative error
max_i |du_i| / sum_j |K_ij w_j| (the gate of the split form)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-6
SPLIT = 1


def _case(seed, N, k, m, n, dist="unif"):
    rng = np.random.default_rng(seed)
    if dist == "unif":
        X = rng.random((N, k))
    else:
        X = rng.standard_normal((N, k))
    w = rng.standard_normal(N)
    amap = rng.choice(N, m, replace=False).astype(np.int32)
    bmap = rng.choice(N, n, replace=False).astype(np.int32)
    umap = rng.permutation(N)[:m].astype(np.int32)
    wmap = rng.permutation(N)[:n].astype(np.int32)
    return X, w, amap, bmap, umap, wmap


def _run(gpu, O, ktype, params, X, w, amap, bmap, umap, wmap, hi=None):
    from ks_gb300 import gsks
    torch = gpu
    N, k = X.shape
    m, n = amap.size, bmap.size
    X2 = O.norms(X)
    okern = dict(params)
    if hi is not None:
        okern.update(hi=hi, hj=hi)
    u_ref = np.zeros(N)
    O.dgsks(O.make_kernel(ktype, **okern), u_ref, umap, X, X2, amap, X, X2, bmap, w, wmap)
    _, cond = O.rows(O.make_kernel(ktype, **okern), np.arange(m, dtype=np.int32), X, X2, amap, X, X2, bmap, w, wmap)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    gk = dict(params)
    if hi is not None:
        hd = t(hi)
        gk.update(hi=hd, hj=hd)
    u = torch.zeros(N, dtype=torch.float64, device="cuda")
    gsks.dgsks_device(gsks.make_kernel(ktype, **gk), m, n, k, u, t(umap), t(X), t(X2), t(amap), t(X), t(X2),
                      t(bmap), t(w), t(wmap), precision=SPLIT, stream=torch.cuda.current_stream(), nxa=N, nxb=N)
    torch.cuda.synchronize()
    assert gsks.device_errors() == 0
    got = u.cpu().numpy()
    return O.errors(got[umap], u_ref[umap], cond=cond)


@pytest.mark.parametrize("shape", [(500, 16, 128, 128), (700, 16, 128, 256), (3000, 8, 300, 1000),
                                   (5000, 64, 1000, 1500), (4000, 3, 513, 700), (4000, 37, 200, 333)])
def test_split_gaussian_uniform(gpu, oracle_mod, shape):
    N, k, m, n = shape
    e = _run(gpu, oracle_mod, 0, dict(scal=-2.0), *_case(1, N, k, m, n))
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e


@pytest.mark.parametrize("ktype,params", [
    (1, dict(scal=1 / 16, cons=1.0, powe=3.0)), (1, dict(scal=0.1, cons=0.1, powe=4.0)),
    (2, {}), (4, dict(scal=0.1, cons=0.1)), (6, dict(cons=1.0)),
])
def test_split_other_kernels(gpu, oracle_mod, ktype, params):
    e = _run(gpu, oracle_mod, ktype, params, *_case(2, 3000, 16, 700, 900))
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e


@pytest.mark.parametrize("ktype", [5, 7])
def test_split_compact_kernels(gpu, oracle_mod, ktype):
    X, w, amap, bmap, umap, wmap = _case(3, 3000, 16, 700, 900)
    e = _run(gpu, oracle_mod, ktype, {}, X * 0.2, w, amap, bmap, umap, wmap)
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e


def test_split_var_bandwidth(gpu, oracle_mod):
    X, w, amap, bmap, umap, wmap = _case(4, 4000, 8, 900, 1100)
    rng = np.random.default_rng(44)
    h = np.exp(rng.uniform(np.log(0.05), np.log(0.5), X.shape[0]))
    e = _run(gpu, oracle_mod, 3, {}, X, w, amap, bmap, umap, wmap, hi=1.0 / h)
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e


@pytest.mark.parametrize("shape", [(3000, 128, 300, 400), (2000, 512, 200, 300), (1500, 1000, 150, 200),
                                   (2500, 80, 260, 390)])
def test_split_gaussian_streamed_k(gpu, oracle_mod, shape):
    """k beyond the target-resident kernel: both operands stream in 64-wide k chunks."""
    N, k, m, n = shape
    e = _run(gpu, oracle_mod, 0, dict(scal=-12.0 / k), *_case(5, N, k, m, n))
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e


def test_split_polynomial_dense_k1024(gpu, oracle_mod):
    """The dense configuration's shape at a small size: N(0, 1/k) points, k = 1024,
    pwr 4.  Every value sits near 1 and sum_j K w_j cancels: the row anchors
    carry the constant part in FP64."""
    X, w, amap, bmap, umap, wmap = _case(6, 1200, 1024, 160, 170, dist="normal")
    e = _run(gpu, oracle_mod, 1, dict(scal=1.0, cons=1.0, powe=4.0), X / np.sqrt(1024), w, amap, bmap, umap, wmap)
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e


@pytest.mark.parametrize("pw", [1, 2, 3, 4])
def test_split_polynomial_on_a_constant(gpu, oracle_mod, pw):
    """The general-stride configuration's polynomial at a reduced size (k = 64,
    uniform [0, 1], scal = 1/64, cons = 1) with weights of zero sum: K = (1 +
    x.y/64)^p varies by a few percent around its mean and sum_j K w_j cancels
    down to that variation.  FP32 rounding of K itself then puts the normwise
    error near 3e-6 (a CPU emulation of such an epilogue: 2.6e-6 to 3.1e-6
    for p = 1..4); the sums around row anchors stay near 1e-7."""
    X, w, amap, bmap, umap, wmap = _case(13, 12000, 64, 2500, 6000)
    w[wmap] -= w[wmap].mean()
    e = _run(gpu, oracle_mod, 1, dict(scal=1 / 64, cons=1.0, powe=float(pw)), X, w, amap, bmap, umap, wmap)
    assert e["normwise"] <= 5e-7 and e["cond_max"] <= 1e-8, e


def test_split_tanh_on_a_constant(gpu, oracle_mod):
    """tanh(x.y/64 + 0.2) on uniform [0, 1]^64 with weights of zero sum: the
    values sit within a few percent of tanh(0.45); summed around per-row
    anchors (addition theorem near the anchor)."""
    X, w, amap, bmap, umap, wmap = _case(14, 12000, 64, 2500, 6000)
    w[wmap] -= w[wmap].mean()
    e = _run(gpu, oracle_mod, 4, dict(scal=1 / 64, cons=0.2), X, w, amap, bmap, umap, wmap)
    assert e["normwise"] <= 5e-7 and e["cond_max"] <= 1e-8, e


def test_split_tanh_saturating(gpu, oracle_mod):
    """tanh(x.y) on N(0, 1) points in k = 16: values across both saturated
    ends, far from the rows' anchors (evaluated directly there)."""
    X, w, amap, bmap, umap, wmap = _case(15, 4000, 16, 800, 1000, dist="normal")
    e = _run(gpu, oracle_mod, 4, dict(scal=1.0, cons=0.0), X, w, amap, bmap, umap, wmap)
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e


def _mixture(seed, N, k, ncl=64, sigma=0.05, dup=0.01):
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-10, 10, (ncl, k))
    lab = rng.integers(0, ncl, N)
    X = centres[lab] + sigma * rng.standard_normal((N, k))
    nd = int(dup * N)
    src = rng.choice(N, nd, replace=False)
    dst = rng.choice(N, nd, replace=False)
    X[dst] = X[src]                       # exact duplicates
    return X


@pytest.mark.parametrize("k", [3, 8, 32, 128, 512])
def test_split_mixture_with_duplicates(gpu, oracle_mod, k):
    """The split-precision configuration's data at a reduced size: 64-component
    Gaussian mixture (centres U[-10,10]^k, sigma 0.05) with 1% exact duplicates;
    Gaussian h = 0.2 and polynomial pwr 2."""
    N, m, n = 6000, 1500, 1500
    X = _mixture(10 + k, N, k)
    rng = np.random.default_rng(20 + k)
    w = rng.standard_normal(N)
    amap = rng.choice(N, m, replace=False).astype(np.int32)
    bmap = rng.choice(N, n, replace=False).astype(np.int32)
    umap = rng.permutation(N)[:m].astype(np.int32)
    wmap = rng.permutation(N)[:n].astype(np.int32)
    e = _run(gpu, oracle_mod, 0, dict(scal=-12.5), X, w, amap, bmap, umap, wmap)
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, ("gaussian", e)
    e = _run(gpu, oracle_mod, 1, dict(scal=1.0 / k, cons=1.0, powe=2.0), X, w, amap, bmap, umap, wmap)
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, ("polynomial", e)


def _separated(seed, N, k, src_box, tgt_box, m, n):
    """Sources in the cube src_box^k, targets in tgt_box^k: every kernel value of
    a narrow Gaussian between them lies far below the FP32 range."""
    rng = np.random.default_rng(seed)
    X = np.empty((N, k))
    half = N // 2
    X[:half] = rng.uniform(*src_box, (half, k))
    X[half:] = rng.uniform(*tgt_box, (N - half, k))
    w = rng.standard_normal(N)
    bmap = rng.choice(half, n, replace=False).astype(np.int32)
    amap = (half + rng.choice(N - half, m, replace=False)).astype(np.int32)
    umap = rng.permutation(N)[:m].astype(np.int32)
    wmap = rng.permutation(N)[:n].astype(np.int32)
    return X, w, amap, bmap, umap, wmap


def test_split_gaussian_below_fp32_range_rescaled(gpu, oracle_mod):
    """K between 1e-41 and 1e-63 (FP64 normal, FP32 zero) with a distance bound
    tight enough for FP32 values: rows are summed relative to their largest value."""
    case = _separated(7, 4000, 3, (0.0, 0.1), (0.9, 1.0), 600, 900)
    e = _run(gpu, oracle_mod, 0, dict(scal=-48.5), *case)
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e


def test_split_gaussian_below_fp32_range_fp64(gpu, oracle_mod):
    """K near 1e-170 with a loose distance bound: those rows go to FP64."""
    case = _separated(8, 4000, 16, (0.0, 0.3), (0.7, 1.0), 500, 700)
    e = _run(gpu, oracle_mod, 0, dict(scal=-100.0), *case)
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e


def test_split_var_bandwidth_narrow(gpu, oracle_mod):
    """Bandwidth products up to 2500 (h down to 0.02): the pairs whose FP32
    value is not accurate enough are recomputed in FP64."""
    X, w, amap, bmap, umap, wmap = _case(9, 4000, 8, 700, 900)
    rng = np.random.default_rng(45)
    h = np.exp(rng.uniform(np.log(0.02), np.log(0.7), X.shape[0]))
    e = _run(gpu, oracle_mod, 3, {}, X, w, amap, bmap, umap, wmap, hi=1.0 / h ** 2)
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e


def test_split_gaussian_rows_partly_below_fp32_range(gpu, oracle_mod):
    """Sources in two clusters, taken cluster by cluster (so that 32-column
    groups are pure); targets near either cluster or far from both.  Near rows
    skip the other cluster's groups (values below the FP32 range, negligible
    against the row); far rows have only such values and are redone in full."""
    rng = np.random.default_rng(12)
    N, k, m, n = 6000, 3, 900, 1200
    X = np.empty((N, k))
    X[:2000] = rng.uniform(0.0, 0.1, (2000, k))
    X[2000:4000] = rng.uniform(0.5, 0.6, (2000, k))
    X[4000:] = rng.uniform(1.4, 1.5, (2000, k))
    w = rng.standard_normal(N)
    bmap = np.concatenate([rng.choice(2000, n // 2, replace=False),
                           2000 + rng.choice(2000, n // 2, replace=False)]).astype(np.int32)
    amap = rng.permutation(np.concatenate([rng.choice(2000, m // 3, replace=False) + o
                                           for o in (0, 2000, 4000)])).astype(np.int32)
    umap = rng.permutation(N)[:m].astype(np.int32)
    wmap = rng.permutation(N)[:n].astype(np.int32)
    e = _run(gpu, oracle_mod, 0, dict(scal=-200.0), X, w, amap, bmap, umap, wmap)
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e
