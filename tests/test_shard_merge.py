"""Row-range sharding of the exhaustive search: the merge of every shard's k best
equals the unsharded k best (ids and distances), checked with the oracle's linear
search per shard on the CPU, and across two gloo ranks (the host-memory exchange the
multi-GPU split uses)."""
import os
import socket

import numpy as np
import pytest

import oracle
from golden_util import materialize
from ngt_gb300.shard import gather_and_merge, merge_topk, shard_ranges


def test_shard_ranges_cover_every_slot():
    for nrows, n in ((5001, 2), (5001, 3), (1_000_001, 8), (300, 4)):
        r = shard_ranges(nrows, n)
        assert len(r) == n
        covered = np.zeros(nrows, bool)
        for b, e in r:
            assert b % 128 == 0 and b <= e <= nrows
            covered[b:e] = True
        assert covered.all()


def _shard_results(path, queries, k, ranges):
    """The oracle's exact linear search restricted to each shard's objects."""
    files = oracle.IndexFiles(path)
    o = oracle.Oracle(files)
    rows = o.prepare(queries)
    ids_l, ds_l, cnt_l = [], [], []
    for b, e in ranges:
        d = np.array([[oracle_dist(o, files, rows[j], files.objects[i]) for i in range(max(b, 1), e)]
                      for j in range(len(queries))], np.float32)
        ids = np.arange(max(b, 1), e, dtype=np.uint32)
        order = np.lexsort((np.broadcast_to(ids, d.shape), d), axis=1)[:, :k]
        ids_l.append(ids[order])
        ds_l.append(np.take_along_axis(d, order, axis=1))
        cnt_l.append(np.full(len(queries), min(k, e - max(b, 1)), np.uint32))
    return ids_l, ds_l, cnt_l


def oracle_dist(o, files, a, b):
    return np.float32(o.lib.oracle_distance(files.otype, files.metric, np.ascontiguousarray(a).ctypes.data,
                                            np.ascontiguousarray(b).ctypes.data, files.dpad))


def test_merge_of_shards_equals_whole_linear_search(tmp_path):
    path, meta, queries, golden = materialize("c1_f32_l2", str(tmp_path))
    q = queries[:20]
    k = 10
    o = oracle.Oracle(oracle.IndexFiles(path))
    wi, wd, wn = o.linear_search(q, k=k)
    for n in (2, 3):
        il, dl, cl = _shard_results(path, q, k, shard_ranges(o.f.nrows, n))
        mi, md, mn = merge_topk(il, dl, cl, k)
        assert np.array_equal(mn, wn)
        assert np.array_equal(mi, wi[:, :k])
        assert np.array_equal(md.view(np.uint32), wd[:, :k].view(np.uint32))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, path, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    q = np.load(os.path.join(path, "q.npy"))
    files = oracle.IndexFiles(path)
    b, e = shard_ranges(files.nrows, world)[rank]
    il, dl, cl = _shard_results(path, q, 10, [(b, e)])
    res = gather_and_merge(il[0], dl[0], cl[0], 10)
    if rank == 0:
        np.savez(out, ids=res[0], d=res[1], n=res[2])
    dist.destroy_process_group()


def test_two_gloo_ranks_merge_through_host_memory(tmp_path):
    import multiprocessing as mp
    path, meta, queries, golden = materialize("c1_f32_l2", str(tmp_path))
    q = queries[:12]
    np.save(os.path.join(path, "q.npy"), q)
    out = str(tmp_path / "merged.npz")
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank, args=(r, 2, port, path, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    m = np.load(out)
    o = oracle.Oracle(oracle.IndexFiles(path))
    wi, wd, wn = o.linear_search(q, k=10)
    assert np.array_equal(m["n"], wn)
    assert np.array_equal(m["ids"], wi[:, :10])
    assert np.array_equal(m["d"].view(np.uint32), wd[:, :10].view(np.uint32))
