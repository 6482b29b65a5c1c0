"""CPU tests of the ONNG construction's oracle: the restatement of `ngt
reconstruct-graph -m S` (GraphReconstructor::reconstructGraph and
adjustPathsEffectively) rebuilds, from the reference's own ANNG, exactly the graph
the reference wrote (every node's ids and distances, in order)."""
import gzip
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = [("onng_f32_l2", 10, 50, 0), ("onng_u8_l2_minedges", 16, 30, 12)]


def _graph(name, fn, tmp_path):
    p = tmp_path / (name + "_" + fn)
    p.write_bytes(gzip.open(os.path.join(GOLDEN, name, fn + ".gz")).read())
    return oracle.read_graph_file(str(p))


@pytest.mark.parametrize("name,outgoing,incoming,min_edges", CASES)
def test_oracle_onng_equals_reference(name, outgoing, incoming, min_edges, tmp_path):
    anng = _graph(name, "anng_grp", tmp_path)
    gold = _graph(name, "grp", tmp_path)
    got = oracle.onng(anng, outgoing, incoming, min_edges)
    assert np.array_equal(got["off"], gold["off"])
    assert np.array_equal(got["ids"], gold["ids"])
    assert np.array_equal(got["dists"].view(np.uint32), gold["dists"].view(np.uint32))
    # the construction really removed and added edges
    assert len(gold["ids"]) != len(anng["ids"])


def test_oracle_onng_planted_mistake_is_caught(tmp_path):
    """A changed reverse-edge count gives a different graph: the comparison above
    is sensitive to the parameters."""
    name, o, i, e = CASES[0]
    anng = _graph(name, "anng_grp", tmp_path)
    gold = _graph(name, "grp", tmp_path)
    got = oracle.onng(anng, o, i - 1, e)
    assert not (np.array_equal(got["off"], gold["off"]) and np.array_equal(got["ids"], gold["ids"]))
