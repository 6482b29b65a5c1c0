"""GPU tests of the ONNG construction (ngtgpu_build_onng): from the reference's ANNG
it writes the reference's ONNG graph file byte for byte; on a graph with hub nodes
(more neighbours than the shared-memory hash holds, more candidates than the
shared-memory sort holds) it equals the oracle's construction."""
import gzip
import os
import shutil

import numpy as np
import pytest

import oracle
from golden_util import materialize

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name,outgoing,incoming,min_edges",
                         [("onng_f32_l2", 10, 50, 0), ("onng_u8_l2_minedges", 16, 30, 12)])
def test_build_onng_writes_the_reference_graph(name, outgoing, incoming, min_edges, tmp_path):
    from ngt_gb300 import build_onng
    path, meta, queries, golden = materialize(name, str(tmp_path))
    anng = str(tmp_path / "anng")
    shutil.copytree(path, anng)
    shutil.copy(os.path.join(GOLDEN, name, "anng_prf"), os.path.join(anng, "prf"))
    with open(os.path.join(anng, "grp"), "wb") as f:
        f.write(gzip.open(os.path.join(GOLDEN, name, "anng_grp.gz")).read())
    out = str(tmp_path / "onng")
    build_onng(anng, out, outgoing, incoming, min_edges)
    want = gzip.open(os.path.join(GOLDEN, name, "grp.gz")).read()
    assert open(os.path.join(out, "grp"), "rb").read() == want
    prf = oracle.read_property(out)
    assert prf["GraphType"] == "ONNG"
    # the target must not exist (the reference refuses too)
    from ngt_gb300 import NativeError
    with pytest.raises(NativeError, match="exists"):
        build_onng(anng, out, outgoing, incoming, min_edges)


def _write_graph(path, n, lists):
    with open(path, "wb") as f:
        f.write(np.uint64(n).tobytes())
        f.write(b"-")
        for i in range(1, n):
            ids, ds = lists[i]
            f.write(b"+")
            f.write(np.uint32(len(ids)).tobytes())
            rec = np.empty((len(ids), 2), np.uint32)
            rec[:, 0] = ids
            rec[:, 1] = np.asarray(ds, np.float32).view(np.uint32)
            f.write(rec.tobytes())
        f.write(np.uint32(0).tobytes())            # an empty prevsize vector


def test_build_onng_with_hubs_equals_oracle(tmp_path):
    from ngt_gb300 import build_onng
    rng = np.random.default_rng(5)
    n = 6001                                       # slots: the dummy 0 and nodes 1..6000
    lists = [None]
    for i in range(1, n):
        # 24 edges sorted by (distance, id); every node but node 1 has node 1 among them
        nb = rng.choice(np.arange(2, n), 24, replace=False)
        nb = nb[nb != i][:23]
        nb = np.concatenate([[1], nb]) if i != 1 else rng.choice(np.arange(2, n), 24, replace=False)
        d = rng.random(len(nb)).astype(np.float32) * 10
        if i != 1:
            d[0] = np.float32(0.001 * (i % 97))
        order = np.lexsort((nb, d))
        lists.append((nb[order].astype(np.uint32), d[order]))
    anng = tmp_path / "anng"
    anng.mkdir()
    _write_graph(str(anng / "grp"), n, lists)
    (anng / "prf").write_text("Dimension\t6\nGraphType\tANNG\nIncomingEdge\t24\nOutgoingEdge\t6\n")
    g = oracle.read_graph_file(str(anng / "grp"))
    # node 1 gets a reverse edge from every other node: more neighbours than the 4096 of
    # the shared-memory hash, and more candidates than the shared-memory sort holds
    assert sum(1 in lists[i][0] for i in range(2, n)) > 4096
    want = oracle.onng(g, 6, 24, 0)
    out = str(tmp_path / "onng")
    build_onng(str(anng), out, -1, -1, 0)           # outgoing / incoming from the property file
    got = oracle.read_graph_file(os.path.join(out, "grp"))
    assert np.array_equal(got["off"], want["off"])
    assert np.array_equal(got["ids"], want["ids"])
    assert np.array_equal(got["dists"].view(np.uint32), want["dists"].view(np.uint32))
