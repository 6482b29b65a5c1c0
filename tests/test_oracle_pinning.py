"""Pins the oracle (the CPU restatement in oracle/) to the reference.

The golden vectors under tests/golden/ were produced by the unmodified
reference NGT build (see tests/golden/make_golden.py).  The oracle must agree
with them bit for bit on integer-valued data, and within float rounding on
the float metrics, before it is trusted as the checker of the CUDA library.
"""
import ctypes
import ctypes.util
import os
import re

import numpy as np
import pytest

import oracle
from golden_util import fixture_names, is_integer_fixture, materialize


@pytest.fixture(scope="module")
def workdir(tmp_path_factory):
    return str(tmp_path_factory.mktemp("golden_idx"))


@pytest.mark.parametrize("name", fixture_names())
def test_oracle_matches_reference_golden(name, workdir):
    path, meta, queries, golden = materialize(name, workdir)
    o = oracle.Oracle(oracle.IndexFiles(path))
    exact = is_integer_fixture(name)
    for i, s in enumerate(meta["settings"]):
        nq, k = s["nq"], s["k"]
        gi, gd, gc = golden["ids_%d" % i], golden["dist_%d" % i], golden["count_%d" % i]
        if s["op"] == "linear":
            ids, ds, n = o.linear_search(queries[:nq], k=k, threads=4)
        elif s["op"] == "graph_refine":
            ids, ds, n = o.search_refined(queries[:nq], k=k, epsilon=s["epsilon"], expansion=s["edge_size"],
                                          mode="read_only" if s["mode"] == "ro" else "updatable", threads=4)
        elif s["op"] in ("range", "graph_acc"):
            # range search: the radius in the edge column; expected accuracy: the epsilon
            # comes from the index's AccuracyTable
            eps, radius = s["epsilon"], -1.0
            if s["op"] == "range":
                radius = s["edge_size"]
            else:
                eps = oracle.epsilon_from_accuracy(oracle.read_property(path)["AccuracyTable"], s["edge_size"])
            ids, ds, n, _ = o.search(queries[:nq], k=k, epsilon=eps, radius=radius,
                                     mode="read_only" if s["mode"] == "ro" else "updatable", threads=4)
        elif s["op"] == "qg":
            # quantized graph: the edge column holds the result expansion
            ids, ds, n, _ = o.qg_search(queries[:nq], k=k, epsilon=s["epsilon"], result_expansion=s["edge_size"],
                                        threads=4)
        else:
            es = -1 if s["edge_size"] is None else s["edge_size"]
            ids, ds, n, _ = o.search(queries[:nq], k=k, epsilon=s["epsilon"], edge_size=es,
                                     mode="read_only" if s["mode"] == "ro" else "updatable", threads=4)
        assert (n == gc).all(), (name, s)
        ids, ds = ids[:, :k], ds[:, :k]          # the golden files keep the first k entries
        if exact:
            # integer data: ids and distances identical to the reference
            assert np.array_equal(ids, gi), (name, s)
            assert np.array_equal(ds.view(np.uint32), gd.view(np.uint32)), (name, s)
        else:
            # float data: AVX-512 lane sums vs scalar sums; distances within 1e-5 relative
            # (absolute floor 1e-6 for the bounded cosine-type distances) and ids equal
            # except across near-ties
            tol = 1e-5 * np.maximum(np.abs(gd), 0.1)
            assert (np.abs(ds - gd) <= tol).mean() > 0.99, (name, s)
            assert (ids == gi).all(1).mean() >= 0.98, (name, s)


def test_oracle_rand_matches_glibc():
    libc = ctypes.CDLL(ctypes.util.find_library("c"))
    if not hasattr(libc, "gnu_get_libc_version"):
        pytest.skip("not glibc")
    for seed in (0, 1, 7, 12345, 2 ** 31 - 5):
        libc.srand(ctypes.c_uint(seed))
        want = np.array([libc.rand() for _ in range(1000)], np.int32)
        assert np.array_equal(oracle.rand_sequence(seed, 1000), want)


# the reference sources, where present (the known answer is parsed from them at test time)
REF_ROOT = os.environ.get("NGT_REFERENCE", "")
REF_README = os.path.join(REF_ROOT, "bin", "ngt", "README.md") if REF_ROOT else ""
REF_DATA = os.path.join(REF_ROOT, "data") if REF_ROOT else ""


def _parse_readme_results():
    """The three top-20 result tables of the `ngt search` example (bin/ngt/README.md:276-358)."""
    text = open(REF_README).read()
    blocks = re.findall(r"Query No\.(\d+)[ \t]*\n[ \t]*Rank\tID\tDistance[ \t]*\n((?:[ \t]*\d+\t\d+\t[\d.]+[ \t]*\n)+)",
                        text)
    out = []
    for _, body in blocks:
        rows = [line.strip().split("\t") for line in body.strip().split("\n")]
        out.append([(int(r[1]), float(r[2])) for r in rows])
    return out


@pytest.mark.skipif(not REF_README or not os.path.exists(REF_README),
                    reason="reference sources not present (set NGT_REFERENCE)")
def test_oracle_linear_search_matches_readme_known_answer(tmp_path):
    """The reference README lists the top-20 of three queries on its 5k uint8 SIFT sample;
    an exhaustive search with the oracle's comparator must reproduce ids and distances
    (graph search at epsilon 0.1 on 5k objects is exact for these queries)."""
    expect = _parse_readme_results()
    assert len(expect) == 3
    base = np.loadtxt(os.path.join(REF_DATA, "sift-dataset-5k.tsv"), delimiter="\t")[:, :128]
    qs = np.loadtxt(os.path.join(REF_DATA, "sift-query-3.tsv"), delimiter="\t")[:, :128]
    idx = tmp_path / "sift"
    idx.mkdir()
    (idx / "prf").write_text("Dimension\t128\nDistanceType\tL2\nObjectType\tInteger-1\nIndexType\tGraph\n")
    oracle.write_objects(str(idx / "obj"), base.astype(np.uint8))
    with open(idx / "grp", "wb") as f:
        f.write(np.uint64(base.shape[0] + 1).tobytes() + b"-" * (base.shape[0] + 1))
    o = oracle.Oracle(oracle.IndexFiles(str(idx)))
    ids, ds, n = o.linear_search(qs.astype(np.float32), k=20)
    for q in range(3):
        got = [(int(i), float(d)) for i, d in zip(ids[q], ds[q])]
        for (gi, gd), (ei, ed) in zip(got, expect[q]):
            assert gi == ei
            assert abs(gd - ed) <= 1e-3 * max(1.0, ed)


@pytest.mark.parametrize("name", fixture_names("qbg"))
def test_oracle_qbg_matches_reference_golden(name, workdir):
    """QBG (qbg_search_index_float): ids, quantized distances and counts identical."""
    path, meta, queries, golden = materialize(name, workdir)
    o = oracle.Oracle(oracle.IndexFiles(os.path.join(path, "global")))
    for i, s in enumerate(meta["settings"]):
        # "qbg": the C API (one step, result expansion); "qbg1" / "qbg2": searchInOneStep /
        # searchInTwoSteps with a refinement expansion (exact re-rank over the object list)
        kw = {} if s["op"] == "qbg" else dict(refinement_expansion=s["result_expansion"], two_step=s["op"] == "qbg2")
        ids, ds, n, _ = o.qbg_search(queries[:s["nq"]], path, k=s["k"], epsilon=s["epsilon"],
                                     blob_epsilon=s["blob_epsilon"], result_expansion=s["result_expansion"],
                                     explored_blobs=s["explored_blobs"], threads=4, **kw)
        gi, gd, gc = golden["ids_%d" % i], golden["dist_%d" % i], golden["count_%d" % i]
        assert np.array_equal(n, gc), (name, s)
        assert np.array_equal(ids[:, :s["width"]], gi), (name, s)
        assert np.array_equal(ds[:, :s["width"]].view(np.uint32), gd.view(np.uint32)), (name, s)
