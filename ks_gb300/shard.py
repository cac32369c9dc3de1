"""Multi-GPU sharding of the kernel summation: one process per GPU.

Target rows are independent, so ``dgsks`` shards by contiguous blocks of
target positions (every rank needs the whole source side); ``dgsks_list``
shards by task, balanced by cost m_t * n_t with the greedy largest-first
assignment the reference's OpenMP list driver uses for its worker queues
(frame/omp_dgsks_list.cpp:347-359).  Each rank accumulates its part into a
zero copy of u; one sum all-reduce over the process group then adds every
rank's contributions into u on all ranks (the analogue of the reference's
per-thread ``u_local`` merge, frame/omp_dgsks_list.cpp:407-414).  For
``dgsks`` with an injective umap the parts touch disjoint entries, so the
reduction only moves data.

``compute`` is the per-rank evaluation; by default the GPU entry points of
``ks_gb300.gsks`` on the rank's current device.
"""
from __future__ import annotations

import heapq

import numpy as np


def partition_rows(m: int, world: int) -> list[tuple[int, int]]:
    """Contiguous, balanced [start, end) blocks of m target positions."""
    base, extra = divmod(m, world)
    out, s = [], 0
    for r in range(world):
        e = s + base + (1 if r < extra else 0)
        out.append((s, e))
        s = e
    return out


def partition_tasks(a_off, b_off, world: int) -> list[np.ndarray]:
    """Tasks to ranks, largest cost first, each to the least loaded rank
    (ties to the lower rank); every rank's tasks in ascending order."""
    a_off = np.asarray(a_off, dtype=np.int64)
    b_off = np.asarray(b_off, dtype=np.int64)
    cost = np.diff(a_off) * np.diff(b_off)
    order = sorted(range(cost.size), key=lambda t: (-int(cost[t]), t))
    heap = [(0, r) for r in range(world)]
    owned: list[list[int]] = [[] for _ in range(world)]
    for t in order:
        load, r = heapq.heappop(heap)
        owned[r].append(t)
        heapq.heappush(heap, (load + int(cost[t]), r))
    return [np.array(sorted(x), dtype=np.int64) for x in owned]


def sub_lists(a_off, a_idx, b_off, b_idx, tasks, u_idx=None, w_idx=None):
    """CSR lists of the given tasks (re-based offsets)."""
    a_off = np.asarray(a_off)
    b_off = np.asarray(b_off)
    u_idx = a_idx if u_idx is None else u_idx
    w_idx = b_idx if w_idx is None else w_idx
    out = {}
    for name, off, idx in (("a", a_off, a_idx), ("u", a_off, u_idx), ("b", b_off, b_idx), ("w", b_off, w_idx)):
        parts = [np.asarray(idx[off[t]:off[t + 1]]) for t in tasks]
        out[name + "_idx"] = (np.concatenate(parts) if parts else np.zeros(0)).astype(np.int32)
        if name in ("a", "b"):
            out[name + "_off"] = np.concatenate([[0], np.cumsum([p.size for p in parts])]).astype(np.int32)
    return out


def _allreduce_sum(delta, group):
    import torch
    import torch.distributed as dist
    t = delta if isinstance(delta, torch.Tensor) else torch.from_numpy(delta)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t


def _gpu_dgsks(ker, m, n, k, u, umap, XA, XA2, amap, XB, XB2, bmap, w, wmap, precision):
    import torch
    from . import gsks
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a)).cuda() if not isinstance(a, torch.Tensor) else a.cuda()
    ud = t(u)
    gsks.dgsks_device(ker, m, n, k, ud, t(umap), t(XA), None if XA2 is None else t(XA2), t(amap), t(XB),
                      None if XB2 is None else t(XB2), t(bmap), t(w), t(wmap), precision=precision,
                      stream=torch.cuda.current_stream(), nxa=int(XA.shape[0]), nxb=int(XB.shape[0]))
    torch.cuda.synchronize()
    return ud.cpu().numpy()


def sharded_dgsks(ker, u, umap, XA, XA2, amap, XB, XB2, bmap, w, wmap, rank: int, world: int,
                  group=None, compute=None, precision: int = 0):
    """u[umap[i]] += sum_j K(XA[amap[i]], XB[bmap[j]]) w[wmap[j]] over all ranks'
    target blocks; u (numpy, host) holds the full result on every rank."""
    m, n, k = int(amap.size), int(bmap.size), int(XA.shape[1])
    s, e = partition_rows(m, world)[rank]
    delta = np.zeros_like(u)
    if e > s:
        if compute is None:
            delta = _gpu_dgsks(ker, e - s, n, k, delta, umap[s:e], XA, XA2, amap[s:e], XB, XB2, bmap, w, wmap,
                               precision)
        else:
            compute(ker, delta, np.ascontiguousarray(umap[s:e]), XA, XA2, np.ascontiguousarray(amap[s:e]),
                    XB, XB2, bmap, w, wmap)
    if world > 1:
        delta = _allreduce_sum(delta, group).numpy()
    u += delta
    return u


def sharded_dgsks_list(kers, u, a_off, a_idx, b_off, b_idx, XA, XA2, XB, XB2, w, rank: int, world: int,
                       u_idx=None, w_idx=None, group=None, compute=None):
    """dgsks_list over the tasks this rank owns (partition_tasks), then one sum
    all-reduce; kers: one descriptor per task."""
    mine = partition_tasks(a_off, b_off, world)[rank]
    sub = sub_lists(a_off, a_idx, b_off, b_idx, mine, u_idx, w_idx)
    delta = np.zeros_like(u)
    if mine.size:
        sk = [kers[t] for t in mine]
        if compute is None:
            from . import gsks
            gsks.dgsks_list(sk[0], delta, sub["a_off"], sub["a_idx"], sub["b_off"], sub["b_idx"], XA, XA2, XB,
                            XB2, w, u_idx=sub["u_idx"], w_idx=sub["w_idx"], kers=sk)
        else:
            compute(sk, delta, sub)
    if world > 1:
        delta = _allreduce_sum(delta, group).numpy()
    u += delta
    return u
