"""GPU tests of the serving loop (continuous batching, ngtgpu_server_*).

Requests of different sizes and parameters are submitted from several
threads while earlier ones are on the GPU; each request's results must be
exactly what the same queries return alone through the batched kernel (it
handles every query independently), and latencies must be measured.
"""
import threading

import numpy as np
import pytest

from golden_util import materialize

pytestmark = pytest.mark.gpu
KERNEL_BATCHED = 1


@pytest.fixture(scope="module")
def index_path(tmp_path_factory):
    path, meta, queries, golden = materialize("c1_f32_l2", str(tmp_path_factory.mktemp("serving")))
    return path, queries


@pytest.mark.parametrize("kernel", [1, 3])
def test_results_in_the_mix_equal_results_alone(index_path, kernel):
    from ngt_gb300 import Index, Server
    path, queries = index_path
    rng = np.random.default_rng(7)
    reqs = []
    start = 0
    for _ in range(60):
        n = int(rng.integers(1, 48))
        q = queries[start % 900: start % 900 + n]
        start += n
        reqs.append((q, int(rng.choice([5, 10, 20, 100])), float(rng.choice([0.02, 0.05, 0.1, 0.15, 0.2]))))
    with Index(path, read_only=True) as ix:
        alone = [ix.batch_search(q, k=k, epsilon=e, kernel=kernel) for q, k, e in reqs]
        with Server(ix, max_batch=256, inflight=3, max_k=128, kernel=kernel) as srv:
            tickets = [None] * len(reqs)

            def submitter(part):
                for i in part:
                    q, k, e = reqs[i]
                    tickets[i] = srv.submit(q, k=k, epsilon=e)

            threads = [threading.Thread(target=submitter, args=(range(t, len(reqs), 3),)) for t in range(3)]
            for t in threads:
                t.start()
            for t in threads:
                t.join()
            for i, (q, k, e) in enumerate(reqs):
                ids, ds, n, lat = srv.wait(tickets[i])
                ai, ad, an = alone[i]
                assert np.array_equal(n, an), i
                for j in range(len(q)):
                    assert np.array_equal(ids[j, :n[j]], ai[j, :an[j]]), (i, j)
                    assert np.array_equal(ds[j, :n[j]], ad[j, :an[j]]), (i, j)
                assert lat > 0.0


def test_server_rejects_bad_requests(index_path):
    from ngt_gb300 import Index, NativeError, Server
    path, queries = index_path
    with Index(path, read_only=True) as ix:
        with Server(ix, max_batch=32, inflight=2, max_k=16) as srv:
            with pytest.raises(NativeError, match="request size"):
                srv.submit(queries[:40], k=10)
            with pytest.raises(NativeError, match="maximum"):
                srv.submit(queries[:4], k=40)
            t = srv.submit(queries[:4], k=10)
            ids, ds, n, lat = srv.wait(t)
            assert (n == 10).all()


@pytest.mark.parametrize("two_step,refine", [(False, False), (True, True), (False, True)])
def test_qbg_results_in_the_mix_equal_results_alone(tmp_path, two_step, refine):
    """The serving loop over a QBG index: requests with different k, epsilon, blob
    epsilon, expansion and explored blobs / probes, submitted from several threads
    while others run, each equal to the same queries searched alone."""
    from ngt_gb300 import QBGIndex, QBGServer
    path, meta, queries, golden = materialize("qbg_u8_l2_d64", str(tmp_path))
    rng = np.random.default_rng(11)
    reqs = []
    for _ in range(40):
        n = int(rng.integers(1, 24))
        s0 = int(rng.integers(0, len(queries) - n))
        reqs.append((queries[s0:s0 + n], int(rng.choice([5, 10, 20])), float(rng.choice([0.02, 0.1, 0.2])),
                     float(rng.choice([0.0, 0.05])), float(rng.choice([1.0, 2.0, 3.0])), int(rng.choice([8, 16, 32]))))
    with QBGIndex(path) as ix:
        alone = [ix.batch_search(q, k=k, epsilon=e, blob_epsilon=b, result_expansion=x, explored_blobs=p,
                                 two_step=two_step, refine=refine) for q, k, e, b, x, p in reqs]
        with QBGServer(ix, max_batch=128, inflight=3, max_k=64, two_step=two_step, refine=refine) as srv:
            tickets = [None] * len(reqs)

            def submitter(part):
                for i in part:
                    q, k, e, b, x, p = reqs[i]
                    tickets[i] = srv.submit(q, k=k, epsilon=e, blob_epsilon=b, result_expansion=x, explored_blobs=p)

            threads = [threading.Thread(target=submitter, args=(range(t, len(reqs), 3),)) for t in range(3)]
            for t in threads:
                t.start()
            for t in threads:
                t.join()
            for i in range(len(reqs)):
                ids, ds, n, lat = srv.wait(tickets[i])
                ai, ad, an = alone[i]
                assert np.array_equal(n, an), i
                for j in range(len(n)):
                    assert np.array_equal(ids[j, :n[j]], ai[j, :an[j]]), (i, j)
                    assert np.array_equal(ds[j, :n[j]].view(np.uint32), ad[j, :an[j]].view(np.uint32)), (i, j)
                assert lat > 0.0


@pytest.mark.parametrize("kernel", [0, 3])
def test_qg_results_in_the_mix_equal_results_alone(tmp_path, kernel):
    """The serving loop over a quantized graph: requests with different size,
    epsilon and result expansion, submitted from several threads, each equal to the
    same queries searched alone (and so to ngtqg_search_index_float)."""
    from ngt_gb300 import QGServer, QuantizedIndex
    path, meta, queries, golden = materialize("qg_f32_l2_d32", str(tmp_path))
    rng = np.random.default_rng(13)
    reqs = []
    for _ in range(40):
        n = int(rng.integers(1, 24))
        s0 = int(rng.integers(0, len(queries) - n))
        reqs.append((queries[s0:s0 + n], int(rng.choice([5, 10, 20])), float(rng.choice([0.0, 0.05, 0.1])),
                     float(rng.choice([1.0, 2.0, 3.0]))))
    with QuantizedIndex(path, zero_based_numbering=False) as ix:
        alone = [ix.batch_search(q, size=k, epsilon=e, result_expansion=x, kernel=kernel) for q, k, e, x in reqs]
        with QGServer(ix, max_batch=128, inflight=3, max_k=64, kernel=kernel) as srv:
            tickets = [None] * len(reqs)

            def submitter(part):
                for i in part:
                    q, k, e, x = reqs[i]
                    tickets[i] = srv.submit(q, k=k, epsilon=e, result_expansion=x)

            threads = [threading.Thread(target=submitter, args=(range(t, len(reqs), 3),)) for t in range(3)]
            for t in threads:
                t.start()
            for t in threads:
                t.join()
            for i in range(len(reqs)):
                ids, ds, n, lat = srv.wait(tickets[i])
                ai, ad, an = alone[i]
                assert np.array_equal(n, an), i
                for j in range(len(n)):
                    assert np.array_equal(ids[j, :n[j]], ai[j, :an[j]]), (i, j)
                    assert np.array_equal(ds[j, :n[j]].view(np.uint32), ad[j, :an[j]].view(np.uint32)), (i, j)
                assert lat > 0.0


def test_deadline_and_cancel(index_path):
    """A request that cannot be launched within its admission deadline completes
    unlaunched with an error; a waiting request can be withdrawn; the others are
    served as usual."""
    from ngt_gb300 import Index, NativeError, Server
    path, queries = index_path
    with Index(path, read_only=True) as ix:
        ai, ad, an = ix.batch_search(queries[:8], k=10, epsilon=0.1, kernel=KERNEL_BATCHED)
        with Server(ix, max_batch=64, inflight=1, max_k=16) as srv:
            # a deadline of a nanosecond has passed before the dispatcher can look at it
            t = srv.submit(queries[:8], k=10, deadline_ms=1e-6)
            with pytest.raises(NativeError, match="deadline exceeded"):
                srv.wait(t)
            # the server-wide default, then back to none
            srv.set_deadline(1e-6)
            t = srv.submit(queries[:8], k=10)
            with pytest.raises(NativeError, match="deadline exceeded"):
                srv.wait(t)
            srv.set_deadline(0)
            # withdraw requests queued behind busy work: cancel() says whether each
            # was still waiting; the withdrawn ones report "cancelled", the others
            # deliver their results
            busy = [srv.submit(queries[:64], k=10, epsilon=0.3) for _ in range(4)]
            tail = [srv.submit(queries[:8], k=10, epsilon=0.1) for _ in range(6)]
            withdrawn = [srv.cancel(t) for t in tail]
            for t in busy:
                srv.wait(t)
            for t, w in zip(tail, withdrawn):
                if w:
                    with pytest.raises(NativeError, match="cancelled"):
                        srv.wait(t)
                else:
                    ids, ds, n, lat = srv.wait(t)
                    assert np.array_equal(n, an)
                    assert np.array_equal(ids[:, :10], ai[:, :10])
            assert any(withdrawn)
            t = srv.submit(queries[:8], k=10, epsilon=0.1)
            ids, ds, n, lat = srv.wait(t)
            assert np.array_equal(ids[:, :10], ai[:, :10])
            with pytest.raises(NativeError, match="unknown ticket"):
                srv.cancel(10 ** 9)
