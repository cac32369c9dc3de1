"""Sharding across processes (one per GPU): partitions, and world_size-2 runs
over gloo on the CPU whose results must equal the unsharded oracle's."""
import os
import socket

import numpy as np
import pytest

from ks_gb300 import shard


def test_partition_rows_covers_and_balances():
    for m, world in [(0, 2), (1, 2), (7, 3), (65536, 8)]:
        parts = shard.partition_rows(m, world)
        assert parts[0][0] == 0 and parts[-1][1] == m
        assert all(parts[i][1] == parts[i + 1][0] for i in range(world - 1))
        sizes = [e - s for s, e in parts]
        assert max(sizes) - min(sizes) <= 1


def test_partition_tasks_is_a_balanced_partition():
    rng = np.random.default_rng(0)
    sa = np.exp(rng.uniform(np.log(32), np.log(4096), 500)).astype(int)
    sb = np.exp(rng.uniform(np.log(32), np.log(4096), 500)).astype(int)
    a_off = np.concatenate([[0], np.cumsum(sa)])
    b_off = np.concatenate([[0], np.cumsum(sb)])
    for world in (1, 2, 4, 8):
        parts = shard.partition_tasks(a_off, b_off, world)
        allt = np.sort(np.concatenate(parts))
        assert np.array_equal(allt, np.arange(500))
        cost = sa * sb
        loads = [cost[p].sum() for p in parts]
        # greedy largest-first: no rank exceeds the mean by more than one task
        assert max(loads) <= cost.sum() / world + cost.max()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_world_size_2_gloo_matches_unsharded(oracle_mod, tmp_path):
    import torch.multiprocessing as mp
    import _shard_worker as W
    O = oracle_mod
    mp.spawn(W.run, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    # dgsks: every rank holds the full result
    X, w, amap, bmap, umap, wmap = W.case()
    X2 = O.norms(X)
    u_ref = np.full(X.shape[0], 0.25)
    O.dgsks(O.make_kernel(0, scal=-1.5), u_ref, umap, X, X2, amap, X, X2, bmap, w, wmap)
    for r in range(2):
        u = np.load(os.path.join(tmp_path, f"dgsks_{r}.npy"))
        assert O.errors(u, u_ref)["normwise"] <= 1e-13
    # dgsks_list with u entries shared across tasks of different ranks
    X, w, a_off, a_idx, b_off, b_idx, specs = W.list_case()
    X2 = O.norms(X)
    kers = [O.make_kernel(t, **p) for t, p in specs]
    u_ref = np.zeros(X.shape[0])
    O.dgsks_list(kers[0], u_ref, a_off, a_idx, a_idx, b_off, b_idx, b_idx, X, X2, X, X2, w, kers=kers)
    u0 = np.load(os.path.join(tmp_path, "list_0.npy"))
    u1 = np.load(os.path.join(tmp_path, "list_1.npy"))
    assert np.array_equal(u0, u1)
    assert O.errors(u0, u_ref)["normwise"] <= 1e-13
