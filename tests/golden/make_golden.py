"""Generates the golden fixtures under tests/golden/ by running the reference.

Each fixture is a small NGT index built by the unmodified reference CLI
(oracle/_ref/ngt, compiled from the reference sources by `make -C oracle ref`)
over seeded synthetic data, plus the reference's own search results for a set
of (k, epsilon, edge_size, open mode) settings, obtained through the
reference C API by oracle/_ref/ref_dump.  Only this script needs the
reference; the tests read the committed files.

Stored per fixture (tests/golden/<name>/):
  prf               the index property file, verbatim
  grp.gz, tre.gz    the graph and tree files, gzip-compressed
  obj.gz            the object file, unless it is regenerated from the seeds
                    (meta.json "regenerate_obj": true, sha256 recorded)
  qg.tar.gz         for quantized-graph fixtures: the files of <index>/qg that a
                    QG search reads (prf, qr, rqcb, grp, local-*/obj), built by
                    `qbg create-qg` + `qbg build-qg` (oracle/_ref/qbg)
  qbg.tar.gz        for quantized-blob-graph fixtures (no prf/grp/tre/obj.gz of
                    their own): the files of the QBG index directory a search
                    reads (prf, qr, rqcb, grp, local-*/obj, global/{prf,obj,grp,tre}),
                    built by `qbg create` + `qbg append` + `qbg build`
  meta.json         generator, shapes, seeds, the ngt create options
  golden.npz        queries seed + per-setting ids / distances / counts

usage: python tests/golden/make_golden.py [fixture ...]
"""
from __future__ import annotations

import gzip
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tarfile
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from ngt_gb300 import synthetic  # noqa: E402
import oracle  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")

# name -> spec.  "gen": (generator, kwargs) for base and queries; "create": ngt create options.
FIXTURES = {
    "c1_f32_l2": dict(
        base=("clipped_exponential", dict(n=5000, dim=128, seed=1)),
        query=("clipped_exponential", dict(n=1000, dim=128, seed=2)),
        create="-d 128 -o f -D 2 -E 10 -S 40 -i t", regenerate_obj=True, otype="f",
        settings=[("graph", 10, 0.1, None, "ro"), ("graph", 10, 0.0, None, "ro"), ("graph", 20, 0.2, None, "ro"),
                  ("graph", 10, 0.3, None, "ro"), ("graph", 10, 0.1, 0, "ro"), ("graph", 10, 0.1, -2, "ro"),
                  ("graph", 10, 0.1, 10, "ro"), ("graph", 10, 0.1, None, "rw"), ("graph", 100, 0.1, None, "ro:200"),
                  ("graph", 100, 0.1, None, "rw:200"), ("linear", 10, 0.0, None, "ro"),
                  ("linear", 100, 0.0, None, "ro:200")]),
    "c1_f32_l2_onng": dict(
        base=("clipped_exponential", dict(n=5000, dim=128, seed=1)),
        query=("clipped_exponential", dict(n=500, dim=128, seed=2)),
        create="-d 128 -o f -D 2 -E 100 -S 0 -e 0.1 -i t", reconstruct="-m S -o 10 -i 100",
        regenerate_obj=True, otype="f",
        settings=[("graph", 10, 0.1, None, "ro"), ("graph", 10, 0.02, None, "ro"), ("graph", 100, 0.1, None, "ro:100")]),
    # ONNG construction (`ngt reconstruct-graph -m S`): the reference's ANNG is kept
    # (anng_grp.gz, anng_prf) so that the GPU construction can rebuild the ONNG from it
    "onng_f32_l2": dict(
        base=("clipped_exponential", dict(n=2000, dim=32, seed=301)),
        query=("clipped_exponential", dict(n=200, dim=32, seed=302)),
        create="-d 32 -o f -D 2 -E 50 -S 0 -e 0.1 -i t", reconstruct="-m S -o 10 -i 50", keep_anng=True,
        regenerate_obj=True, otype="f",
        settings=[("graph", 10, 0.1, None, "ro"), ("graph", 10, 0.02, None, "rw")]),
    "onng_u8_l2_minedges": dict(
        base=("clipped_exponential", dict(n=1500, dim=48, seed=311)),
        query=("clipped_exponential", dict(n=150, dim=48, seed=312)),
        create="-d 48 -o c -D 2 -E 40 -S 0 -e 0.1 -i t", reconstruct="-m S -o 16 -i 30 -E 12", keep_anng=True,
        regenerate_obj=True, otype="c",
        settings=[("graph", 10, 0.1, None, "ro")]),
    "u8_l2": dict(
        base=("clipped_exponential", dict(n=3000, dim=64, seed=31)),
        query=("clipped_exponential", dict(n=300, dim=64, seed=32)),
        create="-d 64 -o c -D 2 -E 10 -S 40 -i t", regenerate_obj=True, otype="c",
        settings=[("graph", 10, 0.1, None, "ro"), ("graph", 10, 0.1, None, "rw"), ("linear", 10, 0.0, None, "ro")]),
    "u8_l1": dict(
        base=("clipped_exponential", dict(n=2000, dim=48, seed=41)),
        query=("clipped_exponential", dict(n=200, dim=48, seed=42)),
        create="-d 48 -o c -D 1 -E 10 -S 40 -i t", regenerate_obj=True, otype="c",
        settings=[("graph", 10, 0.1, None, "ro"), ("linear", 10, 0.0, None, "ro")]),
    "u8_hamming": dict(
        base=("random_bytes", dict(n=2000, dim=32, seed=51, p_one=0.3)),
        query=("random_bytes", dict(n=200, dim=32, seed=52, p_one=0.3)),
        create="-d 32 -o c -D h -E 10 -S 40 -i t", regenerate_obj=True, otype="c",
        settings=[("graph", 10, 0.1, None, "ro"), ("linear", 10, 0.0, None, "ro")]),
    "u8_jaccard": dict(
        base=("random_bytes", dict(n=2000, dim=32, seed=61, p_one=0.3)),
        query=("random_bytes", dict(n=200, dim=32, seed=62, p_one=0.3)),
        create="-d 32 -o c -D j -E 10 -S 40 -i t", regenerate_obj=True, otype="c",
        settings=[("graph", 10, 0.1, None, "ro"), ("linear", 10, 0.0, None, "ro")]),
    "f32_l1": dict(
        base=("gaussian_mixture", dict(n=2000, dim=32, nclusters=16, seed_means=71, seed=72)),
        query=("gaussian_mixture", dict(n=200, dim=32, nclusters=16, seed_means=71, seed=73)),
        create="-d 32 -o f -D 1 -E 10 -S 40 -i t", regenerate_obj=True, otype="f",
        settings=[("graph", 10, 0.1, None, "ro"), ("linear", 10, 0.0, None, "ro")]),
    "f32_cosine": dict(
        base=("gaussian_mixture", dict(n=2000, dim=32, nclusters=16, seed_means=81, seed=82)),
        query=("gaussian_mixture", dict(n=200, dim=32, nclusters=16, seed_means=81, seed=83)),
        create="-d 32 -o f -D c -E 10 -S 40 -i t", regenerate_obj=True, otype="f",
        settings=[("graph", 10, 0.1, None, "ro"), ("linear", 10, 0.0, None, "ro")]),
    "f32_angle": dict(
        base=("gaussian_mixture", dict(n=2000, dim=32, nclusters=16, seed_means=91, seed=92)),
        query=("gaussian_mixture", dict(n=200, dim=32, nclusters=16, seed_means=91, seed=93)),
        create="-d 32 -o f -D a -E 10 -S 40 -i t", regenerate_obj=True, otype="f",
        settings=[("graph", 10, 0.1, None, "ro"), ("linear", 10, 0.0, None, "ro")]),
    "f32_ncosine": dict(
        base=("gaussian_mixture", dict(n=2000, dim=32, nclusters=16, seed_means=101, seed=102)),
        query=("gaussian_mixture", dict(n=200, dim=32, nclusters=16, seed_means=101, seed=103)),
        create="-d 32 -o f -D C -E 10 -S 40 -i t", regenerate_obj=False, otype="f",
        settings=[("graph", 10, 0.1, None, "ro"), ("linear", 10, 0.0, None, "ro")]),
    "f32_nl2": dict(
        base=("gaussian_mixture", dict(n=2000, dim=32, nclusters=16, seed_means=111, seed=112)),
        query=("gaussian_mixture", dict(n=200, dim=32, nclusters=16, seed_means=111, seed=113)),
        create="-d 32 -o f -D E -E 10 -S 40 -i t", regenerate_obj=False, otype="f",
        settings=[("graph", 10, 0.1, None, "ro"), ("linear", 10, 0.0, None, "ro")]),
    "f16_l2": dict(
        base=("clipped_exponential", dict(n=2000, dim=64, seed=131)),
        query=("clipped_exponential", dict(n=200, dim=64, seed=132)),
        create="-d 64 -o h -D 2 -E 10 -S 40 -i t", regenerate_obj=True, otype="h",
        settings=[("graph", 10, 0.1, None, "ro"), ("linear", 10, 0.0, None, "ro")]),
    "f32_l2_graphonly": dict(
        base=("clipped_exponential", dict(n=2000, dim=32, seed=141)),
        query=("clipped_exponential", dict(n=200, dim=32, seed=142)),
        create="-d 32 -o f -D 2 -E 10 -S 40 -i g", regenerate_obj=True, otype="f",
        settings=[("graph", 10, 0.1, None, "ro"), ("graph", 10, 0.1, None, "rw")]),
    "f32_l2_resultsize": dict(
        base=("clipped_exponential", dict(n=2000, dim=32, seed=151)),
        query=("clipped_exponential", dict(n=200, dim=32, seed=152)),
        create="-d 32 -o f -D 2 -E 10 -S 40 -i t", regenerate_obj=True, otype="f",
        prf_set={"EpsilonType": "ResultSize"},
        settings=[("graph", 10, 0.1, None, "ro"), ("graph", 10, 0.2, None, "rw")]),
    # Range search (radius in the edge column, ngt_search_index_as_float's radius) and
    # the C++ API's expected accuracy (accuracy in the edge column; epsilon from the
    # AccuracyTable property, lib/NGT/Index.h:418-486, 1700-1702)
    "f32_l2_acc_range": dict(
        base=("clipped_exponential", dict(n=2000, dim=32, seed=261)),
        query=("clipped_exponential", dict(n=200, dim=32, seed=262)),
        create="-d 32 -o f -D 2 -E 10 -S 40 -i t", regenerate_obj=True, otype="f",
        prf_set={"AccuracyTable": "0:0.62,0.02:0.78,0.05:0.9,0.1:0.97,0.2:0.995,0.3:1"},
        settings=[("range", 100, 0.1, 110.0, "ro"), ("range", 100, 0.1, 130.0, "rw"), ("range", 20, 0.0, 120.0, "ro"),
                  ("graph_acc", 10, 0.1, 0.85, "ro"), ("graph_acc", 10, 0.1, 0.97, "ro"),
                  ("graph_acc", 20, 0.1, 0.995, "rw"), ("graph_acc", 10, 0.1, 0.5, "ro")]),
    # Refinement objects (lib/NGT/Index.h:1146-1236): int8-code objects searched with
    # k x expansion results, re-ranked by exact distances over float refinement objects
    # (robj; `ngt create -R f` empty, then `ngt append -D r` fills objects and refinement
    # objects); the edge column holds the refinement expansion (the C++ API only)
    "qs8_l2_refine": dict(
        base=("gaussian_mixture", dict(n=2000, dim=32, nclusters=16, seed_means=271, seed=272)),
        query=("gaussian_mixture", dict(n=200, dim=32, nclusters=16, seed_means=271, seed=273)),
        create="-d 32 -o qsu8 -R f -D 2 -E 10 -S 40 -i t", append="-D r", regenerate_obj=False, otype="q",
        settings=[("graph_refine", 10, 0.1, 2.0, "ro"), ("graph_refine", 10, 0.05, 4.0, "ro"),
                  ("graph_refine", 20, 0.1, 1.5, "rw"), ("graph", 10, 0.1, None, "ro")]),
    # Scalar-quantized objects (ObjectType QSUInteger-8B): int8 codes
    # rint(x / QuantizationScale x 127.5), the query quantized the same way
    "qs8_l2": dict(
        base=("gaussian_mixture", dict(n=2000, dim=32, nclusters=16, seed_means=191, seed=192)),
        query=("gaussian_mixture", dict(n=200, dim=32, nclusters=16, seed_means=191, seed=193)),
        create="-d 32 -o qsu8 -D 2 -E 10 -S 40 -i t", regenerate_obj=False, otype="q",
        settings=[("graph", 10, 0.1, None, "ro"), ("graph", 10, 0.02, None, "ro"), ("graph", 20, 0.2, None, "rw"),
                  ("linear", 10, 0.0, None, "ro")]),
    # Scalar-quantized objects under the inner product and the normalized cosine: the
    # stored codes are shifted to unsigned (code + 127) and the search compares the
    # signed query codes with them by one integer dot product
    # (ObjectSpaceRepository::isQsint8Quint8, lib/NGT/ObjectSpaceRepository.h:1343-1347;
    # PrimitiveComparator::InnerProductQsint8 / NormalizedCosineSimilarityQsint8,
    # lib/NGT/PrimitiveComparator.h:376-404); the tree compares by the unsigned-byte L2.
    "qs8_ip": dict(
        base=("gaussian_mixture", dict(n=2000, dim=32, nclusters=16, seed_means=281, seed=282)),
        query=("gaussian_mixture", dict(n=200, dim=32, nclusters=16, seed_means=281, seed=283)),
        create="-d 32 -o qsu8 -D i -E 10 -S 40 -i t", append=True, regenerate_obj=False, otype="q",
        settings=[("graph", 10, 0.1, None, "ro"), ("graph", 10, 0.1, None, "rw"), ("graph", 20, 0.2, None, "ro"),
                  ("linear", 10, 0.0, None, "ro")]),
    "qs8_ncosine": dict(
        base=("gaussian_mixture", dict(n=2000, dim=32, nclusters=16, seed_means=291, seed=292)),
        query=("gaussian_mixture", dict(n=200, dim=32, nclusters=16, seed_means=291, seed=293)),
        create="-d 32 -o qsu8 -D C -E 10 -S 40 -i t", regenerate_obj=False, otype="q",
        settings=[("graph", 10, 0.1, None, "ro"), ("graph", 10, 0.1, None, "rw"), ("graph", 20, 0.2, None, "ro"),
                  ("linear", 10, 0.0, None, "ro")]),
    # Quantized graphs (ngtqg_search_index_float); for "qg" settings the edge
    # column holds the result expansion.
    "qg_f32_l2_d32": dict(
        base=("clipped_exponential", dict(n=2000, dim=32, seed=161)),
        query=("clipped_exponential", dict(n=200, dim=32, seed=162)),
        create="-d 32 -o f -D 2 -E 16 -S 40 -i t",
        regenerate_obj=True, otype="f", qg=dict(create="", build="-E 64"),
        settings=[("qg", 10, 0.1, 3.0, "rw"), ("qg", 10, 0.02, 3.0, "rw"), ("qg", 10, 0.1, 0.0, "rw"),
                  ("qg", 20, 0.1, 1.5, "rw"), ("qg", 10, 0.1, 1.0, "rw")]),
    # Inner product: stored as L2 over (D+1)-dimensional rows whose last element is
    # sqrt(MaxMagnitude - |x|^2) (lib/NGT/Index.cpp:455-640).  `ngt create` with a data
    # file stops with "Index is unavailable" for this distance (its createIndex reaches
    # getIndex() on a bare GraphAndTreeIndex, lib/NGT/Index.cpp:189-214,914-930), so the
    # index is created empty and filled by `ngt append`, the path that computes the
    # magnitudes.  The object file holds the augmented rows, so it is stored.
    "f32_ip": dict(
        base=("gaussian_mixture", dict(n=2000, dim=32, nclusters=16, seed_means=201, seed=202)),
        query=("gaussian_mixture", dict(n=200, dim=32, nclusters=16, seed_means=201, seed=203)),
        create="-d 32 -o f -D i -E 10 -S 40 -i t", append=True, regenerate_obj=False, otype="f",
        settings=[("graph", 10, 0.1, None, "ro"), ("graph", 10, 0.1, None, "rw"), ("graph", 20, 0.2, None, "ro"),
                  ("linear", 10, 0.0, None, "ro")]),
    "f32_poincare": dict(
        base=("poincare_ball", dict(n=2000, dim=16, nclusters=16, seed_means=211, seed=212)),
        query=("poincare_ball", dict(n=200, dim=16, nclusters=16, seed_means=211, seed=213)),
        create="-d 16 -o f -D p -E 10 -S 40 -i t", regenerate_obj=True, otype="f",
        settings=[("graph", 10, 0.1, None, "ro"), ("linear", 10, 0.0, None, "ro")]),
    "f32_lorentz": dict(
        base=("lorentz_hyperboloid", dict(n=2000, dim=16, nclusters=16, seed_means=221, seed=222)),
        query=("lorentz_hyperboloid", dict(n=200, dim=16, nclusters=16, seed_means=221, seed=223)),
        create="-d 16 -o f -D l -E 10 -S 40 -i t", regenerate_obj=True, otype="f",
        settings=[("graph", 10, 0.1, None, "ro"), ("linear", 10, 0.0, None, "ro")]),
    "qg_f32_l2_d64_q2": dict(
        base=("clipped_exponential", dict(n=2000, dim=64, seed=171)),
        query=("clipped_exponential", dict(n=200, dim=64, seed=172)),
        create="-d 64 -o f -D 2 -E 16 -S 40 -i t",
        regenerate_obj=True, otype="f", qg=dict(create="-Q 2", build="-Q 2 -E 48"),
        settings=[("qg", 10, 0.1, 3.0, "rw"), ("qg", 10, 0.1, 0.0, "rw")]),
    # The quantized-graph shape of the 1M x 100 angular workload at small scale:
    # unit-normalised Gaussian-cluster vectors of dimension 100 (pseudo-dimension
    # 112, so 56 two-dimensional subspaces of which 6 are zero padding), an ONNG
    # (10 outgoing / 100 incoming edges), rotation by the optimizer's default.
    "qg_f32_l2_d100_q2": dict(
        base=("gaussian_mixture", dict(n=3000, dim=100, nclusters=30, seed_means=231, seed=232, normalize=True)),
        query=("gaussian_mixture", dict(n=200, dim=100, nclusters=30, seed_means=231, seed=233, normalize=True)),
        create="-d 100 -o f -D 2 -E 100 -S 0 -e 0.1 -i t", reconstruct="-m S -o 10 -i 100",
        regenerate_obj=True, otype="f", qg=dict(create="-Q 2", build="-Q 2"),
        settings=[("qg", 10, 0.02, 2.0, "rw"), ("qg", 10, 0.05, 3.0, "rw"), ("qg", 10, 0.1, 2.0, "rw"),
                  ("qg", 10, 0.1, 0.0, "rw")]),
}


# Quantized blob graphs (qbg_search_index_float).  Settings: ("qbg", k, epsilon,
# "expansion:explored_blobs:blob_epsilon", "rw").
# ("qbg1", ...) and ("qbg2", ...) run the reference's searchInOneStep / searchInTwoSteps
# through its C++ API (oracle/_ref/ref_qbg_dump) with "refinement_expansion:probes:blob_epsilon":
# the one-step search judges at most `probes` blobs, the two-step search probes `probes`
# blobs found by the global index; with an expansion >= 1 the k x expansion quantized
# results are re-ranked by exact distances over the object file (refineDistances).
QBG_FIXTURES = {
    "qbg_u8_l2_d32": dict(
        base=("clipped_exponential", dict(n=20000, dim=32, seed=181)),
        query=("clipped_exponential", dict(n=100, dim=32, seed=182)),
        create="-d 32 -D 2 -N 16 -o c", build="-B 1000:10,1000:40,0:200",
        settings=[("qbg", 10, 0.1, "3.0:16:0.0", "rw"), ("qbg", 10, 0.1, "3.0:256:0.0", "rw"),
                  ("qbg", 10, 0.0, "1.0:8:0.05", "rw"), ("qbg", 5, 0.2, "2.0:32:0.1", "rw"),
                  ("qbg", 10, 0.1, "0.5:16:0.0", "rw")]),
    # with its object file (qbg_dir/obj), for the refined and two-step searches
    "qbg_u8_l2_d64": dict(
        base=("clipped_exponential", dict(n=20000, dim=64, seed=251)),
        query=("clipped_exponential", dict(n=100, dim=64, seed=252)),
        create="-d 64 -D 2 -N 32 -o c", build="-B 1000:10,1000:40,0:256", with_obj=True,
        settings=[("qbg", 10, 0.1, "3.0:16:0.0", "rw"), ("qbg2", 10, 0.1, "0.0:8:0.0", "rw"),
                  ("qbg2", 10, 0.1, "3.0:8:0.0", "rw"), ("qbg2", 20, 0.1, "2.0:32:0.05", "rw"),
                  ("qbg1", 10, 0.1, "3.0:16:0.0", "rw"), ("qbg1", 10, 0.05, "1.5:64:0.1", "rw")]),
}


def make_qbg(name: str, spec: dict) -> None:
    out = os.path.join(HERE, name)
    base = gen(spec["base"])
    queries = gen(spec["query"])
    with tempfile.TemporaryDirectory() as tmp:
        tsv = os.path.join(tmp, "base.tsv")
        np.savetxt(tsv, base.astype(np.int64), fmt="%d", delimiter="\t")
        idx = os.path.join(tmp, "idx")
        run([os.path.join(REF, "qbg"), "create"] + spec["create"].split() + [idx])
        run([os.path.join(REF, "qbg"), "append", idx, tsv])
        run([os.path.join(REF, "qbg"), "build"] + spec["build"].split() + [idx])
        os.makedirs(out, exist_ok=True)
        members = ["prf", "qr", "rqcb", "grp"] + sorted(
            "%s/obj" % d for d in os.listdir(idx) if d.startswith("local-")) + [
            "global/prf", "global/obj", "global/grp", "global/tre"] + (["obj"] if spec.get("with_obj") else [])
        with tarfile.open(os.path.join(out, "qbg.tar.gz"), "w:gz") as tf:
            for m in members:
                info = tf.gettarinfo(os.path.join(idx, m), arcname=m)
                info.mtime, info.uid, info.gid, info.uname, info.gname = 0, 0, 0, "", ""
                with open(os.path.join(idx, m), "rb") as fi:
                    tf.addfile(info, fi)
        qf = os.path.join(tmp, "q.f32")
        queries.astype(np.float32).tofile(qf)
        arrays, settings = {}, []
        for i, (op, k, eps, edge, mode) in enumerate(spec["settings"]):
            nq = queries.shape[0]
            dump = os.path.join(tmp, "out%d" % i)
            if op == "qbg":
                run([os.path.join(REF, "ref_dump"), op, idx, qf, str(nq), str(queries.shape[1]), str(k), repr(eps),
                     edge, mode, dump])
                exp = float(edge.split(":")[0])
                w = int(np.float32(k) * np.float32(exp)) if exp >= 1.0 else k
            else:
                e_, b_, be_ = edge.split(":")
                run([os.path.join(REF, "ref_qbg_dump"), "one" if op == "qbg1" else "two", idx, qf, str(nq),
                     str(queries.shape[1]), str(k), repr(eps), be_, b_, e_, dump])
                w = k
            raw = np.fromfile(dump, np.uint8)
            arrays["ids_%d" % i] = raw[:nq * w * 4].view(np.uint32).reshape(nq, w)
            arrays["dist_%d" % i] = raw[nq * w * 4:2 * nq * w * 4].view(np.float32).reshape(nq, w)
            arrays["count_%d" % i] = raw[2 * nq * w * 4:].view(np.uint32)
            e, b, be = edge.split(":")
            settings.append(dict(op=op, k=k, epsilon=eps, result_expansion=float(e), explored_blobs=int(b),
                                 blob_epsilon=float(be), mode=mode, nq=nq, width=w))
        np.savez_compressed(os.path.join(out, "golden.npz"), **arrays)
    meta = dict(name=name, kind="qbg", base=spec["base"], query=spec["query"], create=spec["create"],
                build=spec["build"], settings=settings,
                reference="NGT " + open(os.path.join(REF, "include", "NGT", "version_defs.h")).read().split('"')[-2])
    with open(os.path.join(out, "meta.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print("wrote", out)


def gen(spec):
    name, kw = spec
    return getattr(synthetic, name)(**kw)


def object_rows(x: np.ndarray, otype: str) -> np.ndarray:
    return {"f": np.float32, "c": np.uint8, "h": np.float16}[otype](x) if otype != "f" else x.astype(np.float32)


def run(cmd, **kw):
    r = subprocess.run(cmd, capture_output=True, text=True, **kw)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout


def make(name: str, spec: dict) -> None:
    out = os.path.join(HERE, name)
    base = gen(spec["base"])
    queries = gen(spec["query"])
    with tempfile.TemporaryDirectory() as tmp:
        tsv = os.path.join(tmp, "base.tsv")
        np.savetxt(tsv, base, fmt="%.9g", delimiter="\t")
        idx = os.path.join(tmp, "idx")
        if spec.get("append"):
            run([os.path.join(REF, "ngt"), "create"] + spec["create"].split() + [idx])
            extra = spec["append"].split() if isinstance(spec["append"], str) else []
            run([os.path.join(REF, "ngt"), "append"] + extra + [idx, tsv])
        else:
            run([os.path.join(REF, "ngt"), "create"] + spec["create"].split() + [idx, tsv])
        if spec.get("keep_anng"):
            # the ANNG before the reconstruction: input of the ONNG construction tests
            os.makedirs(out, exist_ok=True)
            shutil.copy(os.path.join(idx, "prf"), os.path.join(out, "anng_prf"))
            with open(os.path.join(idx, "grp"), "rb") as fi, \
                    gzip.GzipFile(os.path.join(out, "anng_grp.gz"), "wb", mtime=0) as fo:
                fo.write(fi.read())
        if "reconstruct" in spec:
            idx2 = os.path.join(tmp, "idx2")
            run([os.path.join(REF, "ngt"), "reconstruct-graph"] + spec["reconstruct"].split() + [idx, idx2])
            idx = idx2
        if "prf_set" in spec:
            prf = oracle.read_property(idx)
            prf.update(spec["prf_set"])
            with open(os.path.join(idx, "prf"), "w") as f:
                for k in sorted(prf):
                    f.write("%s\t%s\n" % (k, prf[k]))
        if "qg" in spec:
            run([os.path.join(REF, "qbg"), "create-qg"] + spec["qg"]["create"].split() + [idx])
            run([os.path.join(REF, "qbg"), "build-qg"] + spec["qg"]["build"].split() + [idx])
        os.makedirs(out, exist_ok=True)
        shutil.copy(os.path.join(idx, "prf"), os.path.join(out, "prf"))
        if "qg" in spec:
            qgdir = os.path.join(idx, "qg")
            members = ["prf", "qr", "rqcb", "grp"] + sorted(
                "%s/obj" % d for d in os.listdir(qgdir) if d.startswith("local-"))
            with tarfile.open(os.path.join(out, "qg.tar.gz"), "w:gz") as tf:
                for m in members:
                    info = tf.gettarinfo(os.path.join(qgdir, m), arcname=m)
                    info.mtime, info.uid, info.gid, info.uname, info.gname = 0, 0, 0, "", ""
                    with open(os.path.join(qgdir, m), "rb") as fi:
                        tf.addfile(info, fi)
        for fn in ("grp", "tre", "obj", "robj"):
            src = os.path.join(idx, fn)
            if fn == "robj" and (not os.path.exists(src) or os.path.getsize(src) <= 8):
                continue
            if not os.path.exists(src) or (fn == "obj" and spec["regenerate_obj"]):
                continue
            with open(src, "rb") as fi, gzip.GzipFile(os.path.join(out, fn + ".gz"), "wb", mtime=0) as fo:
                fo.write(fi.read())
        obj_sha = hashlib.sha256(open(os.path.join(idx, "obj"), "rb").read()).hexdigest()
        if spec["regenerate_obj"]:
            regen = os.path.join(tmp, "obj_regen")
            oracle.write_objects(regen, object_rows(base, spec["otype"]))
            if hashlib.sha256(open(regen, "rb").read()).hexdigest() != obj_sha:
                raise RuntimeError(name + ": regenerated object file differs from the reference's")
        qf = os.path.join(tmp, "q.f32")
        queries.astype(np.float32).tofile(qf)
        arrays = {}
        settings = []
        for i, (op, k, eps, edge, mode) in enumerate(spec["settings"]):
            nq = queries.shape[0]
            if ":" in mode:
                mode, nq = mode.split(":")[0], int(mode.split(":")[1])
            dump = os.path.join(tmp, "out%d" % i)
            run([os.path.join(REF, "ref_dump"), op, idx, qf, str(nq), str(queries.shape[1]), str(k), repr(eps),
                 "x" if edge is None else repr(edge) if op == "qg" else str(edge), mode, dump])
            raw = np.fromfile(dump, np.uint8)
            ids = raw[:nq * k * 4].view(np.uint32).reshape(nq, k)
            ds = raw[nq * k * 4:2 * nq * k * 4].view(np.float32).reshape(nq, k)
            cnt = raw[2 * nq * k * 4:].view(np.uint32)
            arrays["ids_%d" % i], arrays["dist_%d" % i], arrays["count_%d" % i] = ids, ds, cnt
            settings.append(dict(op=op, k=k, epsilon=eps, edge_size=edge, mode=mode, nq=nq))
        np.savez_compressed(os.path.join(out, "golden.npz"), **arrays)
    meta = dict(name=name, base=spec["base"], query=spec["query"], create=spec["create"],
                reconstruct=spec.get("reconstruct"), keep_anng=bool(spec.get("keep_anng")),
                prf_set=spec.get("prf_set"), qg=spec.get("qg"),
                otype=spec["otype"],
                regenerate_obj=spec["regenerate_obj"], obj_sha256=obj_sha, settings=settings,
                reference="NGT " + open(os.path.join(REF, "include", "NGT", "version_defs.h")).read().split('"')[-2])
    with open(os.path.join(out, "meta.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print("wrote", out)


if __name__ == "__main__":
    names = sys.argv[1:] or list(FIXTURES) + list(QBG_FIXTURES)
    for n in names:
        if n in QBG_FIXTURES:
            make_qbg(n, QBG_FIXTURES[n])
        else:
            make(n, FIXTURES[n])
