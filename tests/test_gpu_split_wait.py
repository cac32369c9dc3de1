"""The bounded waits of the split-precision kernel run out, and the library says so.

The test hook gsks_split_test_wait makes the bulk-copy role of every CTA issue
nothing and shortens the wait limit to 1e5 clock cycles: the tensor-core and
epilogue roles then wait for data that never comes.  Every such wait is
bounded; when it gives up the CTA records the timeout, lets nothing in flight
land (nothing was issued), frees its tensor memory and returns.  Nothing
faults and nothing is left waiting.  The synchronous entry points must then
return GSKS_ERR_TIMEOUT and leave the caller's u alone, the asynchronous one
must set bit 1 of the device error flags, and the next normal call must work
(tensor memory was freed) and match the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPLIT = 1
TIMEOUT_BIT = 2
SHORT_WAIT = 100_000          # clock cycles, about 50 us


def _case(O):
    rng = np.random.default_rng(71)
    N, k, m, n = 2000, 16, 300, 400
    X = rng.random((N, k))
    X2 = O.norms(X)
    w = rng.standard_normal(N)
    amap = rng.choice(N, m, replace=False).astype(np.int32)
    bmap = rng.choice(N, n, replace=False).astype(np.int32)
    umap = rng.permutation(N)[:m].astype(np.int32)
    wmap = rng.permutation(N)[:n].astype(np.int32)
    return X, X2, w, amap, bmap, umap, wmap


@pytest.mark.parametrize("ktype,params", [(1, dict(scal=1 / 16, cons=1.0, powe=3.0)), (0, dict(scal=-2.0))])
def test_split_wait_runs_out_is_reported_and_recovers(gpu, oracle_mod, ktype, params):
    from ks_gb300 import gsks
    torch, O = gpu, oracle_mod
    X, X2, w, amap, bmap, umap, wmap = _case(O)
    N = X.shape[0]
    m, n, k = amap.size, bmap.size, X.shape[1]
    ker = lambda: gsks.make_kernel(ktype, **params)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()

    prev = gsks.get_precision()
    gsks.set_precision(SPLIT)
    try:
        assert gsks.device_errors() == 0
        gsks.split_test_wait(SHORT_WAIT, stall=True)
        # synchronous, host arrays: a status, and u as it was
        u = np.full(N, 7.0)
        rc = gsks.dgsks_status(ker(), u, umap, X, X2, amap, X, X2, bmap, w, wmap)
        assert rc == gsks.GSKS_ERR_TIMEOUT, gsks.error_string(rc)
        assert np.all(u == 7.0)
        # synchronous, device arrays: a status
        ud = torch.zeros(N, dtype=torch.float64, device="cuda")
        rc = gsks.dgsks_status(ker(), ud, t(umap), t(X), t(X2), t(amap), t(X), t(X2), t(bmap), t(w), t(wmap))
        assert rc == gsks.GSKS_ERR_TIMEOUT, gsks.error_string(rc)
        # asynchronous: the flag, read once
        gsks.dgsks_device(ker(), m, n, k, ud, t(umap), t(X), t(X2), t(amap), t(X), t(X2), t(bmap), t(w), t(wmap),
                          precision=SPLIT, stream=torch.cuda.current_stream(), nxa=N, nxb=N)
        torch.cuda.synchronize()
        assert gsks.device_errors() & TIMEOUT_BIT
        assert gsks.device_errors() == 0
        # batched form, host arrays: a status, and u as it was
        a_off = np.array([0, 150, m], dtype=np.int32)
        b_off = np.array([0, 250, n], dtype=np.int32)
        u = np.full(N, 7.0)
        with pytest.raises(gsks.GsksError) as ex:
            gsks.dgsks_list(ker(), u, a_off, amap, b_off, bmap, X, X2, X, X2, w, u_idx=umap, w_idx=wmap)
        assert ex.value.code == gsks.GSKS_ERR_TIMEOUT
        assert np.all(u == 7.0)
    finally:
        gsks.split_test_wait(0, stall=False)
        gsks.set_precision(prev)

    # normal operation again: the same context, correct results
    u_ref = np.zeros(N)
    O.dgsks(O.make_kernel(ktype, **params), u_ref, umap, X, X2, amap, X, X2, bmap, w, wmap)
    _, cond = O.rows(O.make_kernel(ktype, **params), np.arange(m, dtype=np.int32), X, X2, amap, X, X2, bmap, w,
                     wmap)
    gsks.set_precision(SPLIT)
    try:
        u = np.zeros(N)
        rc = gsks.dgsks_status(ker(), u, umap, X, X2, amap, X, X2, bmap, w, wmap)
    finally:
        gsks.set_precision(prev)
    assert rc == 0, gsks.error_string(rc)
    e = O.errors(u[umap], u_ref[umap], cond=cond)
    assert e["normwise"] <= 1e-6 and e["cond_max"] <= 1e-6, e
    ud = torch.zeros(N, dtype=torch.float64, device="cuda")
    gsks.dgsks_device(ker(), m, n, k, ud, t(umap), t(X), t(X2), t(amap), t(X), t(X2), t(bmap), t(w), t(wmap),
                      precision=SPLIT, stream=torch.cuda.current_stream(), nxa=N, nxb=N)
    torch.cuda.synchronize()
    assert gsks.device_errors() == 0
    e = O.errors(ud.cpu().numpy()[umap], u_ref[umap], cond=cond)
    assert e["normwise"] <= 1e-6 and e["cond_max"] <= 1e-6, e
