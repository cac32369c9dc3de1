"""Rank body of the world_size-2 sharding tests (gloo, CPU): the oracle stands
in for each rank's GPU evaluation, so the partition and reduction logic of
ks_gb300.shard is what is tested."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def case(seed=3):
    rng = np.random.default_rng(seed)
    N, k, m, n = 2000, 8, 700, 900
    X = rng.random((N, k))
    w = rng.standard_normal(N)
    amap = rng.choice(N, m, replace=False).astype(np.int32)
    bmap = rng.choice(N, n, replace=False).astype(np.int32)
    umap = rng.permutation(N)[:m].astype(np.int32)
    wmap = rng.permutation(N)[:n].astype(np.int32)
    return X, w, amap, bmap, umap, wmap


def list_case(seed=4):
    rng = np.random.default_rng(seed)
    N, k, ntask = 1500, 6, 30
    X = rng.random((N, k))
    w = rng.standard_normal(N)
    sa = rng.integers(0, 200, ntask)
    sb = rng.integers(0, 200, ntask)
    a_idx = np.concatenate([rng.permutation(N)[:s] for s in sa]).astype(np.int32)
    b_idx = np.concatenate([rng.permutation(N)[:s] for s in sb]).astype(np.int32)
    a_off = np.concatenate([[0], np.cumsum(sa)]).astype(np.int32)
    b_off = np.concatenate([[0], np.cumsum(sb)]).astype(np.int32)
    specs = [(0, dict(scal=-0.7)) if t % 3 == 0 else (2, {}) if t % 3 == 1 else
             (1, dict(scal=0.2, cons=1.0, powe=2.0)) for t in range(ntask)]
    return X, w, a_off, a_idx, b_off, b_idx, specs


def run(rank, world, port, out_dir):
    import torch.distributed as dist
    from oracle import oracle as O
    from ks_gb300 import shard
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        O.build()
        X, w, amap, bmap, umap, wmap = case()
        X2 = O.norms(X)
        u = np.full(X.shape[0], 0.25)

        def compute(ker, u_, umap_, XA, XA2, amap_, XB, XB2, bmap_, w_, wmap_):
            O.dgsks(ker, u_, umap_, XA, XA2, amap_, XB, XB2, bmap_, w_, wmap_)

        shard.sharded_dgsks(O.make_kernel(0, scal=-1.5), u, umap, X, X2, amap, X, X2, bmap, w, wmap,
                            rank, world, compute=compute)
        np.save(os.path.join(out_dir, f"dgsks_{rank}.npy"), u)

        X, w, a_off, a_idx, b_off, b_idx, specs = list_case()
        X2 = O.norms(X)
        kers = [O.make_kernel(t, **p) for t, p in specs]
        u = np.zeros(X.shape[0])

        def compute_list(sk, u_, sub):
            O.dgsks_list(sk[0], u_, sub["a_off"], sub["a_idx"], sub["u_idx"], sub["b_off"], sub["b_idx"],
                         sub["w_idx"], X, X2, X, X2, w, kers=sk)

        shard.sharded_dgsks_list(kers, u, a_off, a_idx, b_off, b_idx, X, X2, X, X2, w, rank, world,
                                 compute=compute_list)
        np.save(os.path.join(out_dir, f"list_{rank}.npy"), u)
    finally:
        dist.destroy_process_group()
