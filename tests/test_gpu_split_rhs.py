"""Several right-hand sides in one split-precision sweep (gsks_dgsks_device_rhs
with GSKS_SPLIT_BF16X3, up to four columns): every kernel value is formed once
and multiplied by each weight column.  Checked column by column against the
oracle at the split gate (1e-6 normwise and conditioned), across the kernel
types and the epilogue's paths: the Gaussian fast path, flagged pairs
rechecked by one lane or by a whole warp (k >= 256), rows redone in full
because all their values lie below the FP32 range, the anchored polynomial,
and the Laplace kernel beyond k = 64, whose layout has no room for the extra
weights (one sweep per column there)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPLIT = 1
TOL = 1e-6


def _weights(rng, N, nrhs, zero_sum_over=None):
    w = rng.standard_normal(N * nrhs)
    if zero_sum_over is not None:          # each column sums to zero over the named sources
        for r in range(nrhs):
            idx = zero_sum_over * nrhs + r
            w[idx] -= w[idx].mean()
    return w


def _run(gpu, O, ktype, params, X, w, amap, bmap, umap, wmap, nrhs, hi=None):
    from ks_gb300 import gsks
    torch = gpu
    N, k = X.shape
    m, n = amap.size, bmap.size
    X2 = O.norms(X)
    ok = dict(params)
    gk = dict(params)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    if hi is not None:
        ok.update(hi=hi, hj=hi)
        hd = t(hi)
        gk.update(hi=hd, hj=hd)
    u0 = np.random.default_rng(3).standard_normal(N * nrhs)
    u_ref = u0.copy()
    conds = []
    for r in range(nrhs):
        ur, wr = (umap * nrhs + r).astype(np.int32), (wmap * nrhs + r).astype(np.int32)
        O.dgsks(O.make_kernel(ktype, **ok), u_ref, ur, X, X2, amap, X, X2, bmap, w, wr)
        _, c = O.rows(O.make_kernel(ktype, **ok), np.arange(m, dtype=np.int32), X, X2, amap, X, X2, bmap, w, wr)
        conds.append(c)
    u = t(u0)
    gsks.dgsks_device_rhs(gsks.make_kernel(ktype, **gk), m, n, k, nrhs, u, t(umap), t(X), t(X2), t(amap), t(X),
                          t(X2), t(bmap), t(w), t(wmap), precision=SPLIT, stream=torch.cuda.current_stream(),
                          nxa=N, nxb=N)
    torch.cuda.synchronize()
    assert gsks.device_errors() == 0
    got = u.cpu().numpy()
    out = []
    for r in range(nrhs):
        idx = umap * nrhs + r
        out.append(O.errors(got[idx], u_ref[idx], cond=conds[r] + np.abs(u0[idx])))
    # entries no target names keep their values
    untouched = np.setdiff1d(np.arange(N), umap)
    idx = (untouched[:, None] * nrhs + np.arange(nrhs)[None, :]).ravel()
    assert np.array_equal(got[idx], u0[idx])
    return out


def _case(seed, N, k, m, n, scale=1.0):
    rng = np.random.default_rng(seed)
    X = rng.random((N, k)) * scale
    amap = rng.choice(N, m, replace=False).astype(np.int32)
    bmap = rng.choice(N, n, replace=False).astype(np.int32)
    umap = rng.permutation(N)[:m].astype(np.int32)
    wmap = rng.permutation(N)[:n].astype(np.int32)
    return rng, X, amap, bmap, umap, wmap


CASES = [
    ("gaussian_fast", 0, dict(scal=-2.0), 64, 1.0),
    ("gaussian_flagged", 0, dict(scal=-60.0), 16, 1.0),
    ("laplace", 2, {}, 16, 1.0),
    ("polynomial_anchored", 1, dict(scal=1 / 16, cons=1.0, powe=3.0), 16, 1.0),
    ("polynomial_pow6", 1, dict(scal=0.1, cons=0.5, powe=6.0), 16, 1.0),
    ("tanh", 4, dict(scal=0.1, cons=0.1), 16, 1.0),
    ("quartic", 5, {}, 16, 0.2),
    ("multiquadratic", 6, dict(cons=1.0), 16, 1.0),
    ("epanechnikov", 7, {}, 16, 0.2),
]


@pytest.mark.parametrize("name,ktype,params,k,scale", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("nrhs", [2, 4])
def test_split_rhs_kernels(gpu, oracle_mod, name, ktype, params, k, scale, nrhs):
    rng, X, amap, bmap, umap, wmap = _case(70 + ktype, 3000, k, 700, 900, scale)
    w = _weights(rng, X.shape[0], nrhs)
    for r, e in enumerate(_run(gpu, oracle_mod, ktype, params, X, w, amap, bmap, umap, wmap, nrhs)):
        assert e["normwise"] <= TOL and e["cond_max"] <= TOL, (r, e)


def test_split_rhs_var_bandwidth_flagged(gpu, oracle_mod):
    rng, X, amap, bmap, umap, wmap = _case(81, 4000, 8, 700, 900)
    h = np.exp(rng.uniform(np.log(0.02), np.log(0.7), X.shape[0]))
    w = _weights(rng, X.shape[0], 3)
    for r, e in enumerate(_run(gpu, oracle_mod, 3, {}, X, w, amap, bmap, umap, wmap, 3, hi=1.0 / h ** 2)):
        assert e["normwise"] <= TOL and e["cond_max"] <= TOL, (r, e)


def test_split_rhs_warp_rechecks_long_rows(gpu, oracle_mod):
    """k = 300: flagged pairs rechecked by a whole warp per pair."""
    rng, X, amap, bmap, umap, wmap = _case(82, 2500, 300, 300, 400)
    w = _weights(rng, X.shape[0], 4)
    for r, e in enumerate(_run(gpu, oracle_mod, 0, dict(scal=-2.0), X, w, amap, bmap, umap, wmap, 4)):
        assert e["normwise"] <= TOL and e["cond_max"] <= TOL, (r, e)


def test_split_rhs_rows_below_fp32_range(gpu, oracle_mod):
    """Targets far from every source under a narrow Gaussian: all values below
    the FP32 range, so every row is redone in full for all its columns."""
    rng = np.random.default_rng(83)
    N, k, m, n = 4000, 3, 500, 700
    X = np.empty((N, k))
    X[: N // 2] = rng.uniform(0.0, 0.1, (N // 2, k))
    X[N // 2:] = rng.uniform(0.9, 1.0, (N - N // 2, k))
    bmap = rng.choice(N // 2, n, replace=False).astype(np.int32)
    amap = (N // 2 + rng.choice(N - N // 2, m, replace=False)).astype(np.int32)
    umap = rng.permutation(N)[:m].astype(np.int32)
    wmap = rng.permutation(N)[:n].astype(np.int32)
    w = _weights(rng, N, 3)
    for r, e in enumerate(_run(gpu, oracle_mod, 0, dict(scal=-48.5), X, w, amap, bmap, umap, wmap, 3)):
        assert e["normwise"] <= TOL and e["cond_max"] <= TOL, (r, e)


def test_split_rhs_polynomial_zero_sum_columns(gpu, oracle_mod):
    """The anchored polynomial with every weight column summing to zero: the
    FP64 anchor term per column carries the constant part."""
    rng, X, amap, bmap, umap, wmap = _case(84, 12000, 64, 1500, 5000)
    w = _weights(rng, X.shape[0], 4, zero_sum_over=wmap)
    out = _run(gpu, oracle_mod, 1, dict(scal=1 / 64, cons=1.0, powe=3.0), X, w, amap, bmap, umap, wmap, 4)
    for r, e in enumerate(out):
        assert e["normwise"] <= 5e-7 and e["cond_max"] <= 1e-8, (r, e)


def test_split_rhs_laplace_streamed_k(gpu, oracle_mod):
    """Laplace at k = 80: the streamed layout with the table has no room for the
    extra weights; the columns are swept one after another (same results)."""
    rng, X, amap, bmap, umap, wmap = _case(85, 2500, 80, 260, 390)
    w = _weights(rng, X.shape[0], 2)
    for r, e in enumerate(_run(gpu, oracle_mod, 2, {}, X, w, amap, bmap, umap, wmap, 2)):
        assert e["normwise"] <= TOL and e["cond_max"] <= TOL, (r, e)
