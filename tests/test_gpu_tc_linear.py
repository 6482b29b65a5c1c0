"""Exhaustive search with the tensor-core pre-selection (tc_linear.cu) through the C ABI.

The approximate scores are checked against numpy on the same bf16-rounded
inputs (exactly on integer-valued data, where every product and partial sum is
an integer below 2^24); the searches against the reference's own linear-search
results of the golden fixtures (ObjectSpaceRepository::linearSearch,
lib/NGT/ObjectSpaceRepository.h:860-922) and, on Gaussian-cluster data of the
precision-path shape, against an FP64 exhaustive ground truth.
"""
import os

import numpy as np
import pytest

from golden_util import materialize

pytestmark = pytest.mark.gpu

FLOAT_LINEAR = ["c1_f32_l2", "f32_cosine", "f32_angle", "f32_ncosine", "f32_nl2"]


@pytest.fixture(scope="module")
def workdir(tmp_path_factory):
    return str(tmp_path_factory.mktemp("gpu_tc"))


def _bf16(x):
    """Round float32 to bf16 (round to nearest even), returned as float64."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def _linear_settings(meta):
    return [(i, s) for i, s in enumerate(meta["settings"]) if s["op"] == "linear"]


def _object_rows(path):
    import oracle
    f = oracle.IndexFiles(path)
    return f, f.objects


def test_scores_exact_on_integer_data(workdir):
    from ngt_gb300 import Index
    path, meta, queries, golden = materialize("c1_f32_l2", workdir)
    f, obj = _object_rows(path)
    x = obj[:, :128].astype(np.float64)
    with Index(path, read_only=True) as ix:
        s = ix.tc_scores(queries[:300])
    q = queries[:300].astype(np.float64)
    ref = q @ x[1:].T - 0.5 * (x[1:] ** 2).sum(1)[None, :]
    assert np.isneginf(s[:, 0]).all()
    assert np.array_equal(s[:, 1:], ref.astype(np.float32))


@pytest.mark.parametrize("name", ["f32_cosine", "f32_ncosine", "f32_nl2"])
def test_scores_float_metrics(name, workdir):
    from ngt_gb300 import Index
    path, meta, queries, golden = materialize(name, workdir)
    with Index(path, read_only=True) as ix:
        rows = ix.convert_queries(queries[:100]).view(np.float32)
        s = ix.tc_scores(queries[:100])
    f, obj = _object_rows(path)
    x = obj[1:].astype(np.float32)
    d = x.shape[1]
    qb, xb = _bf16(rows[:, :d]), _bf16(x)
    dot = qb @ xb.T
    x64 = x.astype(np.float64)
    n2 = (x64 ** 2).sum(1)
    if name == "f32_cosine":
        ref = dot / np.sqrt(n2)[None, :]
    elif name == "f32_nl2":
        ref = dot - 0.5 * n2[None, :]
    else:
        ref = dot
    tol = 1e-5 * np.abs(ref).max() + 1e-6
    assert np.abs(s[:, 1:] - ref).max() <= tol


@pytest.mark.parametrize("first_rows", [0, 256])
@pytest.mark.parametrize("name", FLOAT_LINEAR)
def test_linear_search_matches_reference(name, first_rows, workdir):
    """Both the dense-only path (0: every row of these indexes is scored densely)
    and the threshold filter (256 dense rows) return the reference's results."""
    from ngt_gb300 import Index
    path, meta, queries, golden = materialize(name, workdir)
    for i, s in _linear_settings(meta):
        nq, k = s["nq"], s["k"]
        gi, gd, gc = golden["ids_%d" % i], golden["dist_%d" % i], golden["count_%d" % i]
        with Index(path, read_only=True) as ix:
            ids, ds, n, status = ix.linear_search_tc(queries[:nq], k=k, candidates=max(64, 4 * k),
                                                     first_rows=first_rows)
        assert (status == 0).all()
        assert np.array_equal(n, gc)
        if name == "c1_f32_l2":
            assert np.array_equal(ids, gi) and np.array_equal(ds.view(np.uint32), gd.view(np.uint32))
        else:
            # float metrics: the reference sums with AVX lanes; distances within
            # 1e-5 relative (floor 0.1), ids equal except across near-ties
            tol = 1e-5 * np.maximum(np.abs(gd), 0.1)
            assert (np.abs(ds - gd) <= tol).mean() > 0.99, name
            assert (ids == gi).all(1).mean() >= 0.98, name


def test_linear_search_equals_plain_linear_search(workdir):
    """Ids and distances equal the plain GPU linear search bit for bit."""
    from ngt_gb300 import Index
    path, meta, queries, golden = materialize("f32_cosine", workdir)
    with Index(path, read_only=True) as ix:
        ids, ds, n, status = ix.linear_search_tc(queries[:50], k=20, candidates=128, first_rows=128)
        for j in range(50):
            r = ix.linear_search(queries[j], k=20)
            assert [o.id for o in r] == list(ids[j, : n[j]])
            assert np.array_equal(np.array([o.distance for o in r], np.float32), ds[j, : n[j]])


def test_query_batches_and_repeats(workdir):
    """More queries than one batch (8192): every copy of a query gets the same result."""
    from ngt_gb300 import Index
    path, meta, queries, golden = materialize("c1_f32_l2", workdir)
    reps = np.tile(queries[:100], (90, 1))            # 9000 queries
    with Index(path, read_only=True) as ix:
        ids, ds, n, status = ix.linear_search_tc(reps, k=10, candidates=64, first_rows=512)
    assert (status == 0).all()
    gi = golden["ids_10"][:100]
    for r in range(90):
        assert np.array_equal(ids[r * 100:(r + 1) * 100], gi)


def _cluster_index(tmp, n=20000, dim=768, nq=200, seed=21):
    """Gaussian-cluster float rows (64 means ~ N(0,1), sigma 0.5), L2-normalised,
    written as a NormalizedCosine index; queries from the same mixture."""
    from ngt_gb300.graph_build import write_index
    rng = np.random.default_rng(seed)
    means = rng.standard_normal((64, dim)).astype(np.float32)
    x = means[rng.integers(0, 64, n)] + 0.5 * rng.standard_normal((n, dim)).astype(np.float32)
    q = means[rng.integers(0, 64, nq)] + 0.5 * rng.standard_normal((nq, dim)).astype(np.float32)
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    path = os.path.join(tmp, "clusters")
    ring = np.concatenate([[0], np.arange(2, n + 1), [1]]).astype(np.uint32)[1:]   # node i -> i % n + 1
    offsets = np.concatenate([[0, 0], np.arange(1, n + 1)]).astype(np.int64)
    write_index(path, x, offsets, ring, np.zeros(n, np.float32),
                extra_prf={"DistanceType": "NormalizedCosine", "EdgeSizeForSearch": "10"})
    return path, x, q


def test_fp64_ground_truth_on_clusters(workdir):
    """k=100 with 400 candidates on 20,000 x 768 normalised cluster data: every
    returned id is within the FP64 top 100 (ties at the cut allowed)."""
    from ngt_gb300 import Index
    path, x, q = _cluster_index(workdir)
    qn = q.astype(np.float64) / np.linalg.norm(q.astype(np.float64), axis=1, keepdims=True)
    d64 = 1.0 - qn @ x.astype(np.float64).T
    kth = np.sort(d64, axis=1)[:, 99]
    with Index(path, read_only=True) as ix:
        ids, ds, n, status = ix.linear_search_tc(q, k=100, candidates=400, first_rows=2048)
    assert (status == 0).all() and (n == 100).all()
    got = np.take_along_axis(d64, ids.astype(np.int64) - 1, axis=1)
    assert (got <= kth[:, None] + 1e-6).all()
    assert (np.diff(ds, axis=1) >= 0).all()


def test_low_ids_mostly_removed(workdir):
    """An index whose first 8,000 ids are removed except 40: the dense first part holds
    fewer valid rows than the candidates, so every query's threshold is still -inf in
    the first filtered parts.  The parts are planned so that no candidate list
    overflows (status 0), and the results equal the plain GPU linear search."""
    from ngt_gb300 import Index
    from ngt_gb300.graph_build import write_index
    from ngt_gb300.synthetic import clipped_exponential
    n, dim = 20000, 64
    x = clipped_exponential(n, dim, seed=241)
    q = clipped_exponential(60, dim, seed=242)
    present = np.ones(n + 1, bool)
    present[0] = False
    present[1:8001] = False
    present[1:8001:200] = True
    ids_p = np.nonzero(present)[0]
    deg = np.zeros(n + 1, np.int64)
    deg[ids_p] = 1
    offsets = np.concatenate([[0], np.cumsum(deg)])
    edges = np.roll(ids_p, -1).astype(np.uint32)          # a ring over the present objects
    path = os.path.join(workdir, "removed_low")
    write_index(path, x, offsets, edges, np.ones(len(edges), np.float32), extra_prf={"EdgeSizeForSearch": "10"})
    with open(os.path.join(path, "obj"), "wb") as f:       # removed objects are '-' records
        f.write(np.uint64(n + 1).tobytes())
        f.write(b"-")
        raw = x.view(np.uint8).reshape(n, -1)
        for i in range(1, n + 1):
            f.write(b"+" + raw[i - 1].tobytes() if present[i] else b"-")
    with Index(path, read_only=True) as ix:
        ids, ds, cnt, status = ix.linear_search_tc(q, k=100, candidates=400)
        assert (status == 0).all()
        for j in range(len(q)):
            r = ix.linear_search(q[j], k=100)
            assert [o.id for o in r] == list(ids[j, :cnt[j]])
            assert np.array_equal(np.array([o.distance for o in r], np.float32), ds[j, :cnt[j]])
        assert present[ids[:, :1]].all()


@pytest.mark.parametrize("name", ["c1_f32_l2", "f32_cosine", "f32_ncosine", "f32_ip"])
def test_fp8_scores_return_reference_linear_search(name, workdir):
    """Per-row scaled E4M3 scores (kind::f8f6f4) with an oversampled exact re-rank
    return the reference's recorded linear-search results (ids; distances exact)."""
    from ngt_gb300 import Index
    path, meta, queries, golden = materialize(name, workdir)
    i, s = _linear_settings(meta)[0]
    nq, k = s["nq"], s["k"]
    with Index(path, read_only=True) as ix:
        ids, ds, n, status = ix.linear_search_tc(queries[:nq], k=k, candidates=256, precision="fp8",
                                                 first_rows=256)
    assert (status == 0).all()
    assert np.array_equal(n, golden["count_%d" % i][:nq])
    assert (ids == golden["ids_%d" % i][:nq]).all(1).mean() >= 0.98
    gd = golden["dist_%d" % i][:nq]
    assert (np.abs(ds - gd) <= 1e-5 * np.maximum(np.abs(gd), 0.1)).mean() > 0.99


def test_fp8_and_bf16_agree_with_fp64_ties_on_clusters(workdir):
    """k=100 on 20,000 x 768 normalised cluster data: bf16 (400 candidates) and fp8
    (1,024 candidates) with the FP64 tie check both return exactly the FP64 top 100
    of every query (as a set; ties at the cut decided in FP64)."""
    from ngt_gb300 import Index
    path, x, q = _cluster_index(workdir)
    qn = q.astype(np.float64) / np.linalg.norm(q.astype(np.float64), axis=1, keepdims=True)
    d64 = 1.0 - qn @ x.astype(np.float64).T
    order = np.lexsort((np.broadcast_to(np.arange(d64.shape[1]), d64.shape), d64), axis=1)[:, :100]
    truth = [set((order[j] + 1).tolist()) for j in range(len(q))]
    with Index(path, read_only=True) as ix:
        for prec, C in (("bf16", 400), ("fp8", 1024)):
            ids, ds, n, status = ix.linear_search_tc(q, k=100, candidates=C, first_rows=2048, precision=prec,
                                                     fp64_ties=True)
            assert (status == 0).all() and (n == 100).all(), prec
            agree = np.mean([set(ids[j].tolist()) == truth[j] for j in range(len(q))])
            assert agree == 1.0, (prec, agree)
            assert (np.diff(ds, axis=1) >= 0).all()


@pytest.mark.parametrize("nshards", [2, 3])
def test_row_range_shards_merge_to_the_whole_search(workdir, nshards):
    """The tensor-core search over each shard of a row-range split (the per-GPU part
    of a multi-GPU exhaustive search), merged on the host by (distance, id), equals the
    unsharded search: ids and distances bit for bit."""
    from ngt_gb300 import Index
    from ngt_gb300.shard import merge_topk, shard_ranges
    path, meta, queries, golden = materialize("c1_f32_l2", workdir)
    q = queries[:200]
    with Index(path, read_only=True) as ix:
        wi, wd, wn, ws = ix.linear_search_tc(q, k=10, candidates=64, first_rows=256)
        il, dl, cl = [], [], []
        for b, e in shard_ranges(ix.number_of_objects() + 1, nshards):
            ix._check(ix._lib.ngtgpu_set_tc_row_range(ix._index, b, e, ix._err))
            i, d, n, st = ix.linear_search_tc(q, k=10, candidates=64, first_rows=256)
            assert (st == 0).all()
            assert ((i[:, 0] >= max(b, 1)) & (i[:, 0] < e)).all()
            il.append(i), dl.append(d), cl.append(n)
        ix._check(ix._lib.ngtgpu_set_tc_row_range(ix._index, 0, 0, ix._err))
    mi, md, mn = merge_topk(il, dl, cl, 10)
    assert np.array_equal(mn, wn)
    assert np.array_equal(mi, wi)
    assert np.array_equal(md.view(np.uint32), wd.view(np.uint32))


@pytest.mark.parametrize("precision", ["bf16", "fp8"])
def test_pair_clusters_equal_single_ctas(precision, workdir):
    """The two-CTA cluster form of the score kernel (row tiles 2i and 2i+1 of one
    query tile, the query tile multicast to both) returns the single-CTA results bit
    for bit: 20,001 slots (157 row tiles, the last pair's second tile past the end),
    600 queries (three query tiles, the last ragged), a 2,048-row dense part and the
    filtered parts; and on a 1,000-row fixture with one row tile."""
    from ngt_gb300 import Index
    path, x, _ = _cluster_index(workdir)
    rng = np.random.default_rng(5)
    q = x[rng.integers(0, len(x), 600)] + 0.05 * rng.standard_normal((600, x.shape[1])).astype(np.float32)
    with Index(path, read_only=True) as ix:
        ref = ix.linear_search_tc(q, k=100, candidates=400, first_rows=2048, precision=precision)
        got = ix.linear_search_tc(q, k=100, candidates=400, first_rows=2048, precision=precision, pair=True)
    assert (ref[3] == 0).all()
    for a, b in zip(ref, got):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    path, meta, queries, golden = materialize("c1_f32_l2", workdir)
    with Index(path, read_only=True) as ix:
        ref = ix.linear_search_tc(queries, k=10, candidates=64, first_rows=0, precision=precision)
        got = ix.linear_search_tc(queries, k=10, candidates=64, first_rows=0, precision=precision, pair=True)
    for a, b in zip(ref, got):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_large_query_batches_convert_like_single_queries(workdir):
    """A batch large enough to be converted by several host threads (2,000 x 768
    NormalizedCosine queries: normalised in float, as ObjectSpace::normalize,
    lib/NGT/ObjectSpace.h:356-384) gives every query the row that converting it
    alone gives, bit for bit."""
    from ngt_gb300 import Index
    path, x, q = _cluster_index(workdir)
    big = np.repeat(q, 10, axis=0) * np.linspace(0.5, 2.0, 2000, dtype=np.float32)[:, None]
    with Index(path, read_only=True) as ix:
        rows = ix.convert_queries(big)
        for j in range(0, len(big), 97):
            assert np.array_equal(ix.convert_queries(big[j:j + 1])[0], rows[j]), j


def test_graph_replay_returns_the_direct_results(workdir):
    """With captured launch sequences on, repeated calls (the first captures, the
    rest replay) and calls of other shapes and options return the results of the
    directly launched search, bit for bit."""
    from ngt_gb300 import Index
    path, x, q = _cluster_index(workdir)
    with Index(path, read_only=True) as ix:
        ref = {}
        for nq, prec, pair in ((200, "bf16", False), (64, "bf16", False), (200, "fp8", False), (200, "bf16", True)):
            ref[nq, prec, pair] = ix.linear_search_tc(q[:nq], k=100, candidates=400, first_rows=2048,
                                                      precision=prec, pair=pair)
        ix.set_tc_graphs(True)
        for _ in range(3):
            for (nq, prec, pair), want in ref.items():
                got = ix.linear_search_tc(q[:nq], k=100, candidates=400, first_rows=2048, precision=prec, pair=pair)
                for a, b in zip(want, got):
                    assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (nq, prec, pair)
        ix.set_tc_graphs(False)
        got = ix.linear_search_tc(q[:200], k=100, candidates=400, first_rows=2048)
        for a, b in zip(ref[200, "bf16", False], got):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_empty_batches_and_the_candidate_limit(workdir):
    """An empty query batch returns empty results; more than 4,096 candidates per
    query is refused with an error before any launch, and the handle still serves
    the next call."""
    from ngt_gb300 import Index
    path, meta, queries, golden = materialize("c1_f32_l2", workdir)
    with Index(path, read_only=True) as ix:
        ids, ds, n, status = ix.linear_search_tc(np.zeros((0, queries.shape[1]), np.float32), k=10)
        assert ids.shape == (0, 10) and n.shape == (0,)
        with pytest.raises(Exception):
            ix.linear_search_tc(queries[:4], k=10, candidates=5000)
        ids, ds, n, status = ix.linear_search_tc(queries[:4], k=10, candidates=64)
        assert (status == 0).all() and (n == 10).all()
