"""dgsks_list in the split-precision tensor-core form against the oracle's list
restatement: mixed per-task kernels (Gaussian of several bandwidths, Laplace,
polynomial, variable-bandwidth Gaussian), uneven and empty tasks, separate u
and w maps, host and device arrays, streamed k.

Gate as for the single call: normwise error and the conditioned max-relative
error max_e |du_e| / sum |K w| over the list positions naming u entry e,
both within 1e-6."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-6
SPLIT = 1


def _lists(rng, N, sizes_a, sizes_b):
    a_idx = np.concatenate([rng.permutation(N)[:s] for s in sizes_a]).astype(np.int32)
    b_idx = np.concatenate([rng.permutation(N)[:s] for s in sizes_b]).astype(np.int32)
    a_off = np.concatenate([[0], np.cumsum(sizes_a)]).astype(np.int32)
    b_off = np.concatenate([[0], np.cumsum(sizes_b)]).astype(np.int32)
    return a_off, a_idx, b_off, b_idx


def _cond(O, kers, a_off, a_idx, u_idx, b_off, b_idx, w_idx, X, X2, w, nu):
    """sum over list positions naming each u entry of sum_j |K w| (oracle rows)."""
    cond = np.zeros(nu)
    for t in range(a_off.size - 1):
        a0, a1, b0, b1 = a_off[t], a_off[t + 1], b_off[t], b_off[t + 1]
        if a1 == a0 or b1 == b0:
            continue
        _, c = O.rows(kers[t], np.arange(a1 - a0, dtype=np.int32), X, X2, a_idx[a0:a1], X, X2, b_idx[b0:b1],
                      w, w_idx[b0:b1])
        np.add.at(cond, u_idx[a0:a1], c)
    return cond


def _specs(rng, ntask, k, mix, X=None):
    out = []
    for t in range(ntask):
        c = mix[t % len(mix)]
        if c == "gauss":
            out.append((0, dict(scal=-1.0 / (2 * rng.uniform(0.1, 2.0) ** 2))))
        elif c == "laplace":
            out.append((2, {}))
        elif c == "poly":
            out.append((1, dict(scal=1.0 / k, cons=1.0, powe=float(2 + t % 2))))
        elif c == "varbw":
            out.append((3, {}))
    return out


def _run_list(gpu, O, specs, X, w, a_off, a_idx, u_idx, b_off, b_idx, w_idx, device, hvec=None):
    from ks_gb300 import gsks
    torch = gpu
    N = X.shape[0]
    X2 = O.norms(X)
    kw_o = [dict(p) for _, p in specs]
    kw_g = [dict(p) for _, p in specs]
    hd = torch.from_numpy(hvec).cuda() if (hvec is not None and device) else hvec
    for (t, _), ko, kg in zip(specs, kw_o, kw_g):
        if t == 3:
            ko.update(hi=hvec, hj=hvec)
            kg.update(hi=hd, hj=hd)
    kers_o = [O.make_kernel(t, **p) for (t, _), p in zip(specs, kw_o)]
    kers_g = [gsks.make_kernel(t, **p) for (t, _), p in zip(specs, kw_g)]
    u_ref = np.zeros(N)
    O.dgsks_list(kers_o[0], u_ref, a_off, a_idx, u_idx, b_off, b_idx, w_idx, X, X2, X, X2, w, kers=kers_o)
    cond = _cond(O, kers_o, a_off, a_idx, u_idx, b_off, b_idx, w_idx, X, X2, w, N)
    prev = gsks.get_precision()
    gsks.set_precision(SPLIT)
    try:
        if device:
            t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
            u = torch.zeros(N, dtype=torch.float64, device="cuda")
            gsks.dgsks_list(kers_g[0], u, t(a_off), t(a_idx), t(b_off), t(b_idx), t(X), None, t(X), None, t(w),
                            u_idx=t(u_idx), w_idx=t(w_idx), kers=kers_g)
            torch.cuda.synchronize()
            got = u.cpu().numpy()
        else:
            got = np.zeros(N)
            gsks.dgsks_list(kers_g[0], got, a_off, a_idx, b_off, b_idx, X, X2, X, X2, w, u_idx=u_idx, w_idx=w_idx,
                            kers=kers_g)
        assert gsks.last_launch_count() > 0
    finally:
        gsks.set_precision(prev)
    named = np.unique(u_idx)
    return got, O.errors(got[named], u_ref[named], cond=cond[named])


def test_split_list_mixed_kernels_host(gpu, oracle_mod):
    O = oracle_mod
    rng = np.random.default_rng(11)
    N, k, ntask = 6000, 16, 60
    X = rng.random((N, k)); w = rng.standard_normal(N)
    sa = rng.integers(0, 700, ntask); sb = rng.integers(0, 700, ntask)
    sa[3] = 0; sb[7] = 0                       # empty tasks
    a_off, a_idx, b_off, b_idx = _lists(rng, N, sa, sb)
    u_idx = np.concatenate([rng.permutation(N)[:s] for s in sa]).astype(np.int32)
    w_idx = rng.integers(0, N, b_idx.size).astype(np.int32)
    specs = _specs(rng, ntask, k, ["gauss", "laplace", "poly"])
    got, e = _run_list(gpu, O, specs, X, w, a_off, a_idx, u_idx, b_off, b_idx, w_idx, device=False)
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e
    # deterministic across runs
    got2, _ = _run_list(gpu, O, specs, X, w, a_off, a_idx, u_idx, b_off, b_idx, w_idx, device=False)
    assert np.array_equal(got, got2)


def test_split_list_device_var_bandwidth(gpu, oracle_mod):
    O = oracle_mod
    rng = np.random.default_rng(12)
    N, k, ntask = 5000, 8, 24
    X = rng.random((N, k)); w = rng.standard_normal(N)
    hvec = np.exp(rng.uniform(np.log(2.0), np.log(50.0), N))    # 1 / h^2 for h in [0.14, 0.7]
    sa = rng.integers(1, 900, ntask); sb = rng.integers(1, 1500, ntask)
    a_off, a_idx, b_off, b_idx = _lists(rng, N, sa, sb)
    u_idx = a_idx.copy(); w_idx = b_idx.copy()
    # per task distinct targets: u entries shared across tasks only
    specs = _specs(rng, ntask, k, ["varbw", "gauss"])
    _, e = _run_list(gpu, O, specs, X, w, a_off, a_idx, u_idx, b_off, b_idx, w_idx, device=True, hvec=hvec)
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e


@pytest.mark.parametrize("k", [3, 64, 100])
def test_split_list_log_uniform_sizes(gpu, oracle_mod, k):
    """Task sizes log-uniform in [32, 4096] (the batched workload's distribution,
    fewer tasks), Gaussian h in [0.1, 2], Laplace, polynomial of power 2 or 3."""
    O = oracle_mod
    rng = np.random.default_rng(100 + k)
    N, ntask = 20000, 40
    X = rng.random((N, k)); w = rng.standard_normal(N)
    sa = np.exp(rng.uniform(np.log(32), np.log(4096), ntask)).astype(int)
    sb = np.exp(rng.uniform(np.log(32), np.log(4096), ntask)).astype(int)
    a_off, a_idx, b_off, b_idx = _lists(rng, N, sa, sb)
    u_idx = a_idx.copy(); w_idx = b_idx.copy()
    kinds = ["gauss", "laplace", "poly"] if k > 2 else ["gauss", "poly"]
    specs = _specs(rng, ntask, k, kinds)
    _, e = _run_list(gpu, O, specs, X, w, a_off, a_idx, u_idx, b_off, b_idx, w_idx, device=True)
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e


def test_split_list_rows_below_fp32_range(gpu, oracle_mod):
    """Tasks whose targets lie far from their sources under a narrow Gaussian
    (every value below the FP32 range, nonzero in FP64) beside ordinary tasks:
    such task rows are redone in full after the chunk sums (list_rescue); the
    others keep their FP32 sums."""
    O = oracle_mod
    rng = np.random.default_rng(31)
    k, half = 3, 3000
    X = np.empty((2 * half, k))
    X[:half] = rng.uniform(0.0, 0.1, (half, k))          # sources
    X[half:] = rng.uniform(1.4, 1.5, (half, k))          # far targets
    w = rng.standard_normal(2 * half)
    ntask = 12
    sa = rng.integers(100, 900, ntask); sb = rng.integers(100, 1500, ntask)
    a_parts, b_parts, specs = [], [], []
    for t in range(ntask):
        far = t % 2 == 0
        pool_a = half + rng.permutation(half) if far else rng.permutation(half)
        a_parts.append(pool_a[:sa[t]])
        b_parts.append(rng.permutation(half)[:sb[t]])
        if t % 4 == 0:
            specs.append((0, dict(scal=-60.0)))          # far: K between 2^-585 and 2^-439
        elif t % 4 == 2:
            specs.append((2, {}))                        # far Laplace: ordinary values
        else:
            specs.append((0, dict(scal=-1.0 / (2 * rng.uniform(0.1, 2.0) ** 2))))
    a_idx = np.concatenate(a_parts).astype(np.int32); b_idx = np.concatenate(b_parts).astype(np.int32)
    a_off = np.concatenate([[0], np.cumsum(sa)]).astype(np.int32)
    b_off = np.concatenate([[0], np.cumsum(sb)]).astype(np.int32)
    u_idx = a_idx.copy(); w_idx = b_idx.copy()
    _, e = _run_list(gpu, O, specs, X, w, a_off, a_idx, u_idx, b_off, b_idx, w_idx, device=True)
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e


def test_split_list_more_items_than_ctas_of_uneven_cost(gpu, oracle_mod):
    """Many small tasks and a few large ones: items of very different cost taken
    from the work counter by 152 CTAs."""
    O = oracle_mod
    rng = np.random.default_rng(32)
    N, k, ntask = 30000, 8, 400
    X = rng.random((N, k)); w = rng.standard_normal(N)
    sa = rng.integers(1, 40, ntask); sb = rng.integers(1, 60, ntask)
    sa[:3] = 3000; sb[:3] = 4000
    a_off, a_idx, b_off, b_idx = _lists(rng, N, sa, sb)
    u_idx = a_idx.copy(); w_idx = b_idx.copy()
    specs = _specs(rng, ntask, k, ["gauss", "laplace", "poly"])
    _, e = _run_list(gpu, O, specs, X, w, a_off, a_idx, u_idx, b_off, b_idx, w_idx, device=True)
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e


def test_split_list_polynomial_on_a_constant(gpu, oracle_mod):
    """Polynomial tasks of powers 1..4 (scal 1/k, cons 1, k = 64, uniform [0, 1])
    whose weights sum to zero per task: the values sit within a few percent of
    their mean and sum_j K w_j cancels down to that variation.  Each task's
    rows are summed around their own anchors (the mean of the task's sources),
    with the anchors' part added in FP64 per task."""
    O = oracle_mod
    rng = np.random.default_rng(41)
    N, k, ntask = 20000, 64, 8
    X = rng.random((N, k))
    sa = rng.integers(200, 600, ntask); sb = rng.integers(1000, 3000, ntask)
    a_off, a_idx, b_off, b_idx = _lists(rng, N, sa, sb)
    nb = int(b_off[-1])
    w = rng.standard_normal(max(N, nb))
    w_idx = np.arange(nb, dtype=np.int32)                 # every source position its own weight
    for t in range(ntask):
        blk = slice(b_off[t], b_off[t + 1])
        w[blk] -= w[blk].mean()
    u_idx = np.arange(a_off[-1], dtype=np.int32)          # distinct u entries per task
    specs = [(1, dict(scal=1.0 / k, cons=1.0, powe=float(1 + t % 4))) for t in range(ntask)]
    _, e = _run_list(gpu, O, specs, X, w, a_off, a_idx, u_idx, b_off, b_idx, w_idx, device=True)
    assert e["normwise"] <= 5e-7 and e["cond_max"] <= 1e-8, e


def test_split_list_local_tasks_far_apart(gpu, oracle_mod):
    """Tree-code-like lists: every task's targets and sources come from one
    small cluster (sigma 0.05) of a mixture spread over [-10, 10]^32.  Each
    task is centred and scaled on its own box, so narrow Gaussians and the
    Laplace kernel resolve within the cluster without the error bound of the
    whole data set."""
    O = oracle_mod
    rng = np.random.default_rng(51)
    k, ncl, per = 32, 24, 1200
    centres = rng.uniform(-10, 10, (ncl, k))
    X = (centres[:, None, :] + 0.05 * rng.standard_normal((ncl, per, k))).reshape(-1, k)
    N = X.shape[0]
    w = rng.standard_normal(N)
    sa = rng.integers(200, 800, ncl); sb = rng.integers(300, 900, ncl)
    a_idx = np.concatenate([c * per + rng.permutation(per)[:sa[c]] for c in range(ncl)]).astype(np.int32)
    b_idx = np.concatenate([c * per + rng.permutation(per)[:sb[c]] for c in range(ncl)]).astype(np.int32)
    a_off = np.concatenate([[0], np.cumsum(sa)]).astype(np.int32)
    b_off = np.concatenate([[0], np.cumsum(sb)]).astype(np.int32)
    u_idx = a_idx.copy(); w_idx = b_idx.copy()
    specs = []
    for t in range(ncl):
        specs.append([(0, dict(scal=-12.5)), (2, {}), (0, dict(scal=-200.0))][t % 3])
    _, e = _run_list(gpu, O, specs, X, w, a_off, a_idx, u_idx, b_off, b_idx, w_idx, device=True)
    assert e["normwise"] <= TOL and e["cond_max"] <= TOL, e
