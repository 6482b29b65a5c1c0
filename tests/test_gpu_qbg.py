"""GPU parity of the quantized-blob-graph search (qbg_* C API) with the reference.

The golden vectors came from the reference's qbg_search_index_float over a QBG
index built by `qbg create/append/build`; the GPU results (ids, quantized
distances, counts) must equal them bit for bit.  Further settings are checked
against the oracle, itself pinned to the reference.
"""
import os

import numpy as np
import pytest

import oracle
from golden_util import fixture_names, materialize

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def workdir(tmp_path_factory):
    return str(tmp_path_factory.mktemp("qbg"))


@pytest.mark.parametrize("name", fixture_names("qbg"))
def test_qbg_batch_equals_reference_golden(name, workdir):
    from ngt_gb300 import QBGIndex
    path, meta, queries, golden = materialize(name, workdir)
    with QBGIndex(path) as ix:
        for i, s in enumerate(meta["settings"]):
            # "qbg": the C API's search; "qbg1" / "qbg2": searchInOneStep / searchInTwoSteps with
            # the result expansion as refinement expansion (exact re-rank over the object list)
            kw = {} if s["op"] == "qbg" else dict(two_step=s["op"] == "qbg2", refine=True)
            ids, ds, n = ix.batch_search(queries[:s["nq"]], k=s["k"], epsilon=s["epsilon"],
                                         blob_epsilon=s["blob_epsilon"], result_expansion=s["result_expansion"],
                                         explored_blobs=s["explored_blobs"], **kw)
            gi, gd, gc = golden["ids_%d" % i], golden["dist_%d" % i], golden["count_%d" % i]
            assert np.array_equal(n, gc), (name, s)
            w = ids.shape[1]
            assert np.array_equal(ids, gi[:, :w]), (name, s)
            assert np.array_equal(ds.view(np.uint32), gd[:, :w].view(np.uint32)), (name, s)


@pytest.mark.parametrize("name", fixture_names("qbg"))
def test_qbg_single_query_api_equals_reference_golden(name, workdir):
    from ngt_gb300 import QBGIndex
    path, meta, queries, golden = materialize(name, workdir)
    s = meta["settings"][0]
    with QBGIndex(path) as ix:
        assert ix.dimension == queries.shape[1]
        for j in range(25):
            r = ix.search(queries[j], k=s["k"], epsilon=s["epsilon"], blob_epsilon=s["blob_epsilon"],
                          result_expansion=s["result_expansion"], explored_blobs=s["explored_blobs"])
            assert [o.id for o in r] == list(golden["ids_0"][j, :len(r)])
            assert np.array_equal(np.array([o.distance for o in r], np.float32), golden["dist_0"][j, :len(r)])


@pytest.mark.parametrize("k,eps,beps,expansion,blobs", [(1, 0.1, 0.0, 3.0, 16), (20, 0.05, 0.0, 2.0, 64),
                                                       (10, 0.0, 0.2, 3.0, 8), (10, 0.3, 0.0, 1.5, 400),
                                                       (7, 0.1, 0.05, 0.0, 16), (10, -0.05, 0.0, 3.0, 32)])
def test_qbg_equals_oracle(k, eps, beps, expansion, blobs, workdir):
    from ngt_gb300 import QBGIndex
    name = fixture_names("qbg")[0]
    path, meta, queries, _ = materialize(name, workdir)
    o = oracle.Oracle(oracle.IndexFiles(os.path.join(path, "global")))
    oi, od, on, ob = o.qbg_search(queries, path, k=k, epsilon=eps, blob_epsilon=beps, result_expansion=expansion,
                                  explored_blobs=blobs, threads=8)
    with QBGIndex(path) as ix:
        ids, ds, n, st = ix.batch_search(queries, k=k, epsilon=eps, blob_epsilon=beps, result_expansion=expansion,
                                         explored_blobs=blobs, with_stats=True)
    assert np.array_equal(n, on)
    w = ids.shape[1]
    assert np.array_equal(ids, oi[:, :w])
    assert np.array_equal(ds.view(np.uint32), od[:, :w].view(np.uint32))
    assert np.array_equal(st["visited"], ob)                 # blobs judged
    assert (st["status"] == 0).all()


@pytest.mark.parametrize("two_step", [False, True])
@pytest.mark.parametrize("k,eps,beps,expansion,blobs", [(10, 0.1, 0.0, 3.0, 16), (20, 0.05, 0.05, 2.0, 32),
                                                       (5, 0.1, 0.1, 1.0, 8), (10, 0.1, 0.0, 0.0, 24),
                                                       (1, 0.2, 0.0, 4.0, 64)])
def test_qbg_refined_and_two_step_equal_oracle(k, eps, beps, expansion, blobs, two_step, workdir):
    """The two-step search and the refinement (exact re-rank over the object list)
    against the oracle, itself pinned to the reference's searchInOneStep /
    searchInTwoSteps: ids, exact (or quantized) distances and counts identical."""
    from ngt_gb300 import QBGIndex
    name = "qbg_u8_l2_d64"
    path, meta, queries, _ = materialize(name, workdir)
    o = oracle.Oracle(oracle.IndexFiles(os.path.join(path, "global")))
    oi, od, on, ob = o.qbg_search(queries, path, k=k, epsilon=eps, blob_epsilon=beps, result_expansion=expansion,
                                  explored_blobs=blobs, threads=8, two_step=two_step,
                                  refinement_expansion=expansion)
    with QBGIndex(path) as ix:
        ids, ds, n, st = ix.batch_search(queries, k=k, epsilon=eps, blob_epsilon=beps, result_expansion=expansion,
                                         explored_blobs=blobs, with_stats=True, two_step=two_step, refine=True)
    assert np.array_equal(n, on)
    w = ids.shape[1]
    assert np.array_equal(ids, oi[:, :w])
    assert np.array_equal(ds.view(np.uint32), od[:, :w].view(np.uint32))
    assert np.array_equal(st["visited"], ob)                 # blobs judged
