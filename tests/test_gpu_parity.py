"""GPU parity: the CUDA library against the reference's golden vectors and the oracle.

Every fixture index was built by the reference; its golden results came from
the reference's C API.  The exact-order kernel replays NGT's sequential search,
so on integer-valued data (L2/L1 float or uint8, Hamming, Jaccard, fp16 of
small integers) ids AND distances must be bit-identical to the reference.  On
float metrics the distances are within 1e-5 relative (absolute floor 1e-6 for
the bounded cosine-type distances) and the ids agree except across near-ties.
"""
import numpy as np
import pytest

import oracle
from golden_util import fixture_names, is_integer_fixture, materialize

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def workdir(tmp_path_factory):
    return str(tmp_path_factory.mktemp("gpu_golden"))


def _check(name, s, ids, ds, n, gi, gd, gc):
    k = s["k"]
    assert np.array_equal(n, gc), (name, s, np.nonzero(n != gc)[0][:5])
    ids, ds = ids[:, :k], ds[:, :k]
    valid = np.arange(k)[None, :] < np.minimum(gc, k)[:, None]
    if is_integer_fixture(name):
        assert np.array_equal(np.where(valid, ids, 0), np.where(valid, gi, 0)), name
        assert np.array_equal(np.where(valid, ds, 0).view(np.uint32), np.where(valid, gd, 0).view(np.uint32)), name
    else:
        tol = 1e-5 * np.maximum(np.abs(gd), 0.1)
        assert (np.abs(ds - gd)[valid] <= tol[valid]).mean() > 0.99, name
        assert (np.where(valid, ids, 0) == np.where(valid, gi, 0)).all(1).mean() >= 0.98, name


@pytest.mark.parametrize("name", fixture_names())
def test_batch_search_matches_reference(name, workdir):
    from ngt_gb300 import Index
    path, meta, queries, golden = materialize(name, workdir)
    for i, s in enumerate(meta["settings"]):
        if s["op"] == "qg":
            continue                      # quantized-graph settings: tests/test_gpu_qg.py
        nq, k = s["nq"], s["k"]
        gi, gd, gc = golden["ids_%d" % i], golden["dist_%d" % i], golden["count_%d" % i]
        with Index(path, read_only=(s["mode"] == "ro")) as ix:
            if s["op"] == "graph_acc":
                # the C++ API's expected accuracy: epsilon from the index's AccuracyTable
                ids, ds, n = ix.batch_search_accuracy(queries[:nq], k=k, accuracy=s["edge_size"],
                                                      epsilon=s["epsilon"])
                ids = np.pad(ids, ((0, 0), (0, max(0, k - ids.shape[1]))))
                ds = np.pad(ds, ((0, 0), (0, max(0, k - ds.shape[1]))))
            elif s["op"] == "graph_refine":
                # the C++ API's refinement expansion (the edge column): k x expansion results
                # re-ranked by exact distances over the refinement objects
                ids, ds, n = ix.batch_search_refined(queries[:nq], k=k, expansion=s["edge_size"],
                                                     epsilon=s["epsilon"])
                ids = np.pad(ids, ((0, 0), (0, max(0, k - ids.shape[1]))))
                ds = np.pad(ds, ((0, 0), (0, max(0, k - ds.shape[1]))))
            elif s["op"] == "range":
                # range search: at most k results within the radius (the edge column)
                ids, ds, n = ix.batch_search(queries[:nq], k=k, epsilon=s["epsilon"], radius=s["edge_size"])
                ids = np.pad(ids, ((0, 0), (0, max(0, k - ids.shape[1]))))
                ds = np.pad(ds, ((0, 0), (0, max(0, k - ds.shape[1]))))
            elif s["op"] == "linear":
                res = [ix.linear_search(q, k=k) for q in queries[:nq]]
                n = np.array([len(r) for r in res], np.uint32)
                ids = np.zeros((nq, k), np.uint32)
                ds = np.zeros((nq, k), np.float32)
                for j, r in enumerate(res):
                    ids[j, :len(r)] = [o.id for o in r]
                    ds[j, :len(r)] = [o.distance for o in r]
            else:
                ids, ds, n = ix.batch_search(queries[:nq], k=k, epsilon=s["epsilon"],
                                             edge_size=s["edge_size"] if s["edge_size"] is not None else -1)
                ids = np.pad(ids, ((0, 0), (0, max(0, k - ids.shape[1]))))
                ds = np.pad(ds, ((0, 0), (0, max(0, k - ds.shape[1]))))
        _check(name, s, ids, ds, n, gi, gd, gc)


def test_refined_search_needs_refinement_objects(workdir):
    """An index without refinement objects refuses a refined search with an error."""
    from ngt_gb300 import Index
    from ngt_gb300.base import NativeError
    path, meta, queries, golden = materialize("c1_f32_l2", workdir)
    with Index(path, read_only=True) as ix:
        with pytest.raises(NativeError, match="refinement objects"):
            ix.batch_search_refined(queries[:4], k=10, expansion=2.0)


@pytest.mark.parametrize("name", ["c1_f32_l2", "u8_l2", "qs8_l2"])
def test_single_query_capi_matches_reference(name, workdir):
    """ngt_search_index_as_float one query at a time (the reference's own call)."""
    from ngt_gb300 import Index
    path, meta, queries, golden = materialize(name, workdir)
    s = meta["settings"][0]
    with Index(path, read_only=True) as ix:
        for j in range(20):
            r = ix.search(queries[j], k=s["k"], epsilon=s["epsilon"])
            assert [o.id for o in r] == list(golden["ids_0"][j][: len(r)])
            assert np.array_equal(np.array([o.distance for o in r], np.float32), golden["dist_0"][j][: len(r)])


def test_mixed_parameters_in_one_batch_match_oracle(workdir):
    """Different k / epsilon / edge_size per query in one launch, each as the oracle computes it alone."""
    from ngt_gb300 import Index
    path, meta, queries, _ = materialize("c1_f32_l2", workdir)
    o = oracle.Oracle(oracle.IndexFiles(path))
    rng = np.random.default_rng(5)
    nq = 300
    ks = rng.choice([1, 5, 10, 20, 50], nq)
    eps = rng.choice([0.0, 0.05, 0.1, 0.2], nq).astype(np.float32)
    edges = rng.choice([-1, 0, 10, 20], nq)
    with Index(path, read_only=True) as ix:
        ids, ds, n = ix.batch_search(queries[:nq], k=ks, epsilon=eps, edge_size=edges)
    for j in range(nq):
        oi, od, on, _ = o.search(queries[j:j + 1], k=int(ks[j]), epsilon=float(eps[j]), edge_size=int(edges[j]))
        what = (j, int(ks[j]), float(eps[j]), int(edges[j]))
        assert n[j] == on[0], what
        assert np.array_equal(ids[j, :n[j]], oi[0, :on[0]]), what
        assert np.array_equal(ds[j, :n[j]], od[0, :on[0]]), what


def test_edge_cases(workdir):
    from ngt_gb300 import Index, NativeError
    path, meta, queries, golden = materialize("c1_f32_l2", workdir)
    with Index(path, read_only=True) as ix:
        assert ix.search(queries[0], k=0) == []                       # size 0: nothing
        r = ix.search(queries[0], k=10, epsilon=0.1, radius=0.0)      # radius 0: only exact matches
        assert r == []
        r = ix.search(queries[0], k=10, epsilon=0.1, radius=-1.0)     # negative radius = FLT_MAX
        assert len(r) == 10
        big = ix.linear_search(queries[0], k=6000)                     # k beyond N returns N
        assert len(big) == 5000
        assert [o.id for o in big[:10]] == list(golden["ids_10"][0])
        with pytest.raises(NativeError, match="dimension"):
            ix.search(queries[0][:64], k=10)
        # an object queried against itself: exhaustive search finds it first at distance 0
        f = oracle.IndexFiles(path)
        r = ix.linear_search(f.objects[77, :128].astype(np.float32), k=5)
        assert (r[0].id, r[0].distance) == (77, 0.0)


def test_large_k_and_wide_epsilon_stay_exact(workdir):
    """k=100 at epsilon 0.3 fills the candidate list and the visited table far more; still exact."""
    from ngt_gb300 import Index
    path, meta, queries, _ = materialize("c1_f32_l2", workdir)
    o = oracle.Oracle(oracle.IndexFiles(path))
    with Index(path, read_only=True) as ix:
        ids, ds, n, st = ix.batch_search(queries[:100], k=100, epsilon=0.3, with_stats=True)
    oi, od, on, dc = o.search(queries[:100], k=100, epsilon=0.3, threads=4)
    assert np.array_equal(n, on)
    assert np.array_equal(ids, oi[:, :ids.shape[1]])
    assert np.array_equal(ds, od[:, :ds.shape[1]])
    assert np.array_equal(st["distance_computations"], dc)
    assert (st["status"] & 1 == 0).all()        # no candidate overflow


@pytest.mark.parametrize("mode", ["read_only", "updatable"])
def test_negative_epsilon_matches_oracle(mode, workdir):
    """With epsilon < 0 the exploration radius is tighter than the radius: a
    neighbour joins the results only within both (lib/NGT/Graph.cpp:800-818)."""
    from ngt_gb300 import Index
    path, meta, queries, _ = materialize("c1_f32_l2", workdir)
    o = oracle.Oracle(oracle.IndexFiles(path))
    q = queries[:200]
    for eps in (-0.02, -0.05):
        oi, od, on, _ = o.search(q, k=10, epsilon=eps, mode=mode, threads=8)
        with Index(path, read_only=(mode == "read_only")) as ix:
            ids, ds, n = ix.batch_search(q, k=10, epsilon=eps)
        assert np.array_equal(n, on), eps
        for j in range(len(q)):
            assert np.array_equal(ids[j, :n[j]], oi[j, :n[j]]), (eps, j)
            assert np.array_equal(ds[j, :n[j]].view(np.uint32), od[j, :n[j]].view(np.uint32)), (eps, j)


def test_concurrent_single_query_calls_are_coalesced(workdir):
    """ngt_search_index_as_float from 16 host threads at once (ngtpy's batch_search
    pattern): calls that arrive while a launch runs go together into the next one,
    and every result still equals the reference's."""
    import threading
    from ngt_gb300 import Index
    path, meta, queries, golden = materialize("c1_f32_l2", workdir)
    s = meta["settings"][0]
    nq = 400
    got = [None] * nq
    with Index(path, read_only=True) as ix:
        def worker(part):
            for j in part:
                got[j] = ix.search(queries[j], k=s["k"], epsilon=s["epsilon"])

        threads = [threading.Thread(target=worker, args=(range(t, nq, 16),)) for t in range(16)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        nqc, nlaunch = ix.coalescing_stats()
    assert nqc == nq and 1 <= nlaunch <= nq
    for j in range(nq):
        r = got[j]
        assert [o.id for o in r] == list(golden["ids_0"][j][: len(r)])
        assert np.array_equal(np.array([o.distance for o in r], np.float32), golden["dist_0"][j][: len(r)])
