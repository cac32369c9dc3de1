"""Planned dgsks_list (gsks_list_plan_*): a plan built once evaluates like the
one-shot call, bit for bit; repeated executes replay a CUDA graph and see new
contents of the same buffers; a new buffer is captured afresh."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(torch, seed=21):
    rng = np.random.default_rng(seed)
    N, k, ntask = 5000, 16, 50
    X = rng.random((N, k)); w = rng.standard_normal(N)
    sa = rng.integers(0, 600, ntask); sb = rng.integers(0, 900, ntask)
    a_idx = np.concatenate([rng.permutation(N)[:s] for s in sa]).astype(np.int32)
    b_idx = np.concatenate([rng.permutation(N)[:s] for s in sb]).astype(np.int32)
    a_off = np.concatenate([[0], np.cumsum(sa)]).astype(np.int32)
    b_off = np.concatenate([[0], np.cumsum(sb)]).astype(np.int32)
    specs = [(0, dict(scal=-1.0 / (2 * rng.uniform(0.2, 2.0) ** 2))) if t % 3 == 0 else (2, {}) if t % 3 == 1 else
             (1, dict(scal=1.0 / k, cons=1.0, powe=3.0)) for t in range(ntask)]
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    return dict(N=N, k=k, X=t(X), w=t(w), a_off=t(a_off), a_idx=t(a_idx), b_off=t(b_off), b_idx=t(b_idx),
                specs=specs)


@pytest.mark.parametrize("prec", [0, 1])
def test_plan_matches_one_shot_and_replays(gpu, prec):
    from ks_gb300 import gsks
    torch = gpu
    D = _setup(torch)
    kers = [gsks.make_kernel(t, **p) for t, p in D["specs"]]
    N, k = D["N"], D["k"]
    prev = gsks.get_precision()
    gsks.set_precision(prec)
    try:
        u1 = torch.zeros(N, dtype=torch.float64, device="cuda")
        gsks.dgsks_list(kers[0], u1, D["a_off"], D["a_idx"], D["b_off"], D["b_idx"], D["X"], None, D["X"], None,
                        D["w"], kers=kers)
    finally:
        gsks.set_precision(prev)
    torch.cuda.synchronize()
    plan = gsks.ListPlan(kers[0], D["a_off"], D["a_idx"], D["b_off"], D["b_idx"], k, N, N, N, N, kers=kers,
                         precision=prec, same_pool=True)
    s = torch.cuda.current_stream()
    u2 = torch.zeros(N, dtype=torch.float64, device="cuda")
    plan.execute(u2, D["X"], None, D["X"], None, D["w"], stream=s)      # captured
    torch.cuda.synchronize()
    assert torch.equal(u2, u1)
    plan.execute(u2, D["X"], None, D["X"], None, D["w"], stream=s)      # replayed: accumulates
    torch.cuda.synchronize()
    assert torch.equal(u2, 2 * u1)
    D["w"].mul_(-0.5)                                                    # same buffer, new contents
    u2.zero_()
    plan.execute(u2, D["X"], None, D["X"], None, D["w"], stream=s)
    torch.cuda.synchronize()
    assert torch.equal(u2, -0.5 * u1)
    w2 = D["w"].clone() * -2.0                                          # a new buffer: captured afresh
    u3 = torch.zeros(N, dtype=torch.float64, device="cuda")
    plan.execute(u3, D["X"], None, D["X"], None, w2, stream=s)
    torch.cuda.synchronize()
    assert torch.equal(u3, u1)
    assert plan.errors() == 0
    plan.close()


def test_plan_rejects_bad_lists(gpu):
    from ks_gb300 import gsks
    torch = gpu
    D = _setup(torch, seed=3)
    bad = D["b_idx"].clone()
    bad[5] = D["N"] + 7                                                  # outside the pool
    with pytest.raises(gsks.GsksError):
        gsks.ListPlan(gsks.make_kernel(0, scal=-0.5), D["a_off"], D["a_idx"], D["b_off"], bad, D["k"], D["N"],
                      D["N"], D["N"], D["N"])
