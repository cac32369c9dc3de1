"""gsks_dgsks_device_noalloc: the FP64 kernel summation for callers that may
not allocate device memory (their memory is reserved up front by a pool
allocator, or their loop forbids allocation after start-up).  Its scratch is
a fixed array inside libgsks.so; the test checks, through the C ABI, that two
calls in a row match gsks_dgsks_device and the CPU oracle (sampled rows)
within the FP64 tolerance of the other tests (1e-12), also for the
variable-bandwidth kernel, whose bandwidths come from the descriptor, and
that a too-large m is refused.  Kept in a file of its own that pytest
collects last."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _case(torch, seed, N, k, m, n):
    rng = np.random.default_rng(seed)
    X = rng.random((N, k))
    X2 = (X * X).sum(1)
    w = rng.standard_normal(N)
    amap = rng.choice(N, m, replace=False).astype(np.int32)
    bmap = rng.choice(N, n, replace=False).astype(np.int32)
    umap = rng.permutation(N)[:m].astype(np.int32)
    wmap = rng.permutation(N)[:n].astype(np.int32)
    h = np.exp(rng.uniform(np.log(2.0), np.log(40.0), N))   # var-bandwidth factors
    host = dict(X=X, X2=X2, w=w, amap=amap, bmap=bmap, umap=umap, wmap=wmap, h=h)
    t = lambda a: torch.from_numpy(a).cuda()
    d = {key: t(v) for key, v in host.items()}
    d["host"] = host
    return d


def _oracle_rows(O, ktype, params, d, m, nrows=256):
    """Oracle row sums and sum_j |K w| of up to nrows target positions."""
    g = d["host"]
    rows = np.sort(np.random.default_rng(5).choice(m, min(m, nrows), replace=False)).astype(np.int32)
    kw = dict(params)
    if ktype == 3:
        kw.update(hi=g["h"], hj=g["h"])
    X2 = O.norms(g["X"])
    s, a = O.rows(O.make_kernel(ktype, **kw), rows, g["X"], X2, g["amap"], g["X"], X2, g["bmap"], g["w"], g["wmap"])
    return rows, s, a


def _noalloc(lib, gsks, ker, m, n, k, u, d, stream):
    p = lambda x: C.c_void_p(x.data_ptr())
    return lib.gsks_dgsks_device_noalloc(C.byref(ker), m, n, k, p(u), p(d["umap"]), p(d["X"]), p(d["X2"]),
                                         p(d["amap"]), p(d["X"]), p(d["X2"]), p(d["bmap"]), p(d["w"]),
                                         p(d["wmap"]), C.c_void_p(stream))


@pytest.mark.parametrize("ktype,params,shape", [
    (0, dict(scal=-2.0), (60000, 64, 9000, 20000)),       # chunked sources, many items
    (2, {}, (5000, 16, 1300, 700)),                       # Laplace, tails
    (1, dict(scal=1 / 32, cons=1.0, powe=3.0), (40000, 32, 30000, 2000)),
    (3, {}, (8000, 8, 2500, 3000)),                       # variable bandwidth: hi/hj from the descriptor
])
def test_noalloc_matches_device_entry_two_calls(gpu, oracle_mod, ktype, params, shape):
    from ks_gb300 import gsks
    torch = gpu
    lib = gsks.load()
    lib.gsks_dgsks_device_noalloc.restype = C.c_int
    N, k, m, n = shape
    d = _case(torch, 11 + ktype, N, k, m, n)
    kp = dict(params)
    if ktype == 3:
        kp.update(hi=d["h"], hj=d["h"])
    stream = torch.cuda.current_stream()
    u_ref = torch.zeros(N, dtype=torch.float64, device="cuda")
    gsks.dgsks_device(gsks.make_kernel(ktype, **kp), m, n, k, u_ref, d["umap"], d["X"], d["X2"], d["amap"],
                      d["X"], d["X2"], d["bmap"], d["w"], d["wmap"], stream=stream)
    torch.cuda.synchronize()
    ref = u_ref.cpu().numpy()
    rows, s_or, a_or = _oracle_rows(oracle_mod, ktype, params, d, m)
    umap = d["host"]["umap"]
    for call in range(2):   # the second call finds the first call's scratch contents
        u = torch.zeros(N, dtype=torch.float64, device="cuda")
        rc = _noalloc(lib, gsks, gsks.make_kernel(ktype, **kp), m, n, k, u, d, stream.cuda_stream)
        assert rc == 0, gsks.error_string(rc)
        torch.cuda.synchronize()
        got = u.cpu().numpy()
        assert np.linalg.norm(got - ref) <= TOL * np.linalg.norm(ref), call
        assert gsks.last_launch_count() == 2
        # against the CPU oracle on sampled rows: normwise and conditioned
        e = oracle_mod.errors(got[umap[rows]], s_or, cond=a_or)
        assert e["normwise"] <= TOL and e["cond_max"] <= TOL, (call, e)


def test_noalloc_rejects_m_beyond_scratch(gpu):
    from ks_gb300 import gsks
    torch = gpu
    lib = gsks.load()
    lib.gsks_dgsks_device_noalloc.restype = C.c_int
    d = _case(torch, 3, 100, 4, 10, 10)
    u = torch.zeros(100, dtype=torch.float64, device="cuda")
    # 2^20 + 1 targets need more partial slots than the fixed array holds;
    # the call is refused before any device work.
    rc = _noalloc(lib, gsks, gsks.make_kernel(0, scal=-0.5), (1 << 20) + 1, 10, 4, u, d,
                  torch.cuda.current_stream().cuda_stream)
    assert rc == 11  # GSKS_ERR_TOO_LARGE
    assert float(u.abs().sum()) == 0.0
