"""Split-precision Laplace with nearly coincident points: some targets have a
source at squared distance 1e-6 (k = 16) or 0.05 (k = 64), where the kernel
value exceeds the FP32 range (about 1e40 and 1e56).  The flag rules send such
pairs to the FP64 recheck; a row holding one is redone in FP64 as a whole.
Both the lane-per-pair rechecks (k = 16) and the warp-per-pair ones (k = 64),
single rows and rows with several such pairs, exact duplicates among them, in
one call and through the batched form.  Checked against the oracle at the split
gate (1e-6 normwise and conditioned)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPLIT = 1
TOL = 1e-6


def _near_case(seed, k, d2, N=2500, m=600, n=700, nnear=40):
    rng = np.random.default_rng(seed)
    X = rng.random((N, k))
    amap = rng.choice(N // 2, m, replace=False).astype(np.int32)
    bmap = (N // 2 + rng.choice(N - N // 2, n, replace=False)).astype(np.int32)
    # nnear sources moved next to targets (two of them next to the same target),
    # plus one exact duplicate
    for q in range(nnear):
        i = amap[q if q < nnear - 2 else 0]
        d = rng.standard_normal(k)
        X[bmap[q]] = X[i] + d / np.linalg.norm(d) * np.sqrt(d2)
    X[bmap[nnear]] = X[amap[1]]
    umap = rng.permutation(N)[:m].astype(np.int32)
    wmap = rng.permutation(N)[:n].astype(np.int32)
    w = rng.standard_normal(N)
    return X, w, amap, bmap, umap, wmap


@pytest.mark.parametrize("k,d2", [(16, 1e-6), (64, 0.05)], ids=["k16", "k64"])
def test_split_laplace_values_beyond_fp32(gpu, oracle_mod, k, d2):
    from ks_gb300 import gsks
    torch, O = gpu, oracle_mod
    X, w, amap, bmap, umap, wmap = _near_case(90 + k, k, d2)
    N = X.shape[0]
    m, n = amap.size, bmap.size
    X2 = O.norms(X)
    u0 = np.random.default_rng(1).standard_normal(N)
    ref = u0.copy()
    O.dgsks(O.make_kernel(2), ref, umap, X, X2, amap, X, X2, bmap, w, wmap)
    _, cond = O.rows(O.make_kernel(2), np.arange(m, dtype=np.int32), X, X2, amap, X, X2, bmap, w, wmap)
    assert np.abs(ref - u0).max() > 1e38          # values beyond the FP32 range are present
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    u = t(u0)
    gsks.dgsks_device(gsks.make_kernel(2), m, n, k, u, t(umap), t(X), t(X2), t(amap), t(X), t(X2), t(bmap), t(w),
                      t(wmap), precision=SPLIT, stream=torch.cuda.current_stream(), nxa=N, nxb=N)
    torch.cuda.synchronize()
    assert gsks.device_errors() == 0
    got = u.cpu().numpy()
    assert np.all(np.isfinite(got))
    e = O.errors(got[umap], ref[umap], cond=cond + np.abs(u0[umap]))
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e
    # the same pairs as one task of the batched form
    a_off = np.array([0, m], dtype=np.int32)
    b_off = np.array([0, n], dtype=np.int32)
    prev = gsks.get_precision()
    gsks.set_precision(SPLIT)
    try:
        ul = u0.copy()
        gsks.dgsks_list(gsks.make_kernel(2), ul, a_off, amap, b_off, bmap, X, X2, X, X2, w, u_idx=umap, w_idx=wmap)
    finally:
        gsks.set_precision(prev)
    assert np.all(np.isfinite(ul))
    e = O.errors(ul[umap], ref[umap], cond=cond + np.abs(u0[umap]))
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e
