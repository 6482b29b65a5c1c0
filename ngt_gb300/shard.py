"""Row-range sharding of the exhaustive (linear) search over several GPUs.

A query's exact k nearest objects are the k best, by (distance, id), of the union of
every shard's k best: each GPU searches the objects [begin, end) of its shard
(ngtgpu_set_tc_row_range + ngtgpu_linear_search_tc_*; ids stay global), and one host
merge of the per-shard results gives the whole index's answer -- the same ids and
distances as an unsharded search.  The exchange is nq x k (id, distance) pairs per
shard, gathered through host memory (a gloo process group), with no collective on
the data path of the search itself.
"""
from __future__ import annotations

import numpy as np


def shard_ranges(nrows: int, nshards: int, align: int = 128):
    """[begin, end) object-slot ranges covering slots 1..nrows-1, one per shard, each
    beginning at a multiple of `align` (slot 0 is NGT's unused slot)."""
    if nshards < 1:
        raise ValueError("at least one shard")
    per = -(-nrows // nshards)
    per = -(-per // align) * align
    out = []
    for s in range(nshards):
        b, e = s * per, min(nrows, (s + 1) * per)
        out.append((b, e) if b < e else (0, 0))
    return out


def merge_topk(ids_list, dist_list, count_list, k: int):
    """Per query, the k best (distance, id) pairs over the shards' results.
    ids_list / dist_list: per shard [nq, >=k] arrays; count_list: per shard [nq]."""
    nq = ids_list[0].shape[0]
    out_ids = np.zeros((nq, k), np.uint32)
    out_d = np.zeros((nq, k), np.float32)
    out_n = np.zeros(nq, np.uint32)
    for q in range(nq):
        cand_i, cand_d = [], []
        for ids, ds, cnt in zip(ids_list, dist_list, count_list):
            n = int(cnt[q])
            cand_i.append(ids[q, :n])
            cand_d.append(ds[q, :n])
        ci = np.concatenate(cand_i).astype(np.uint32)
        cd = np.concatenate(cand_d).astype(np.float32)
        order = np.lexsort((ci, cd))[:k]                 # by distance, ties by id
        m = len(order)
        out_ids[q, :m] = ci[order]
        out_d[q, :m] = cd[order]
        out_n[q] = m
    return out_ids, out_d, out_n


def gather_and_merge(ids, dists, counts, k: int, group=None):
    """Every rank's shard results (numpy [nq, k], [nq, k], [nq]) gathered to rank 0
    through a gloo group and merged there; returns the merged result on rank 0 and
    None elsewhere."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    # ids (< 2^32) and float32 distances are exact as float64
    t = torch.from_numpy(np.concatenate([ids.astype(np.float64), dists.astype(np.float64),
                                         counts.astype(np.float64)[:, None]], axis=1))
    bufs = [torch.empty_like(t) for _ in range(world)] if rank == 0 else None
    dist.gather(t, bufs, dst=0, group=group)
    if rank != 0:
        return None
    kk = ids.shape[1]
    il, dl, cl = [], [], []
    for b in bufs:
        a = b.numpy()
        il.append(a[:, :kk].astype(np.int64).astype(np.uint32))
        dl.append(a[:, kk:2 * kk].astype(np.float32))
        cl.append(a[:, 2 * kk].astype(np.uint32))
    return merge_topk(il, dl, cl, k)
