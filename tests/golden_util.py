"""Helpers shared by the tests: materialise a committed golden fixture as an
NGT index directory and load its golden vectors."""
from __future__ import annotations

import gzip
import json
import os
import shutil
import tarfile

import numpy as np

import oracle
from ngt_gb300 import synthetic

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
INTEGER_FIXTURES = {"c1_f32_l2", "c1_f32_l2_onng", "f32_l2_acc_range", "u8_l2", "u8_l1", "u8_hamming", "u8_jaccard", "f16_l2", "qs8_l2", "qs8_ip", "qs8_ncosine", "onng_f32_l2", "onng_u8_l2_minedges",
                    "f32_l2_graphonly", "f32_l2_resultsize", "qg_f32_l2_d32", "qg_f32_l2_d64_q2"}


def fixture_names(kind: str = "graph"):
    """Fixtures of one kind: "graph" (NGT indexes, some with a quantized graph) or "qbg"."""
    out = []
    for d in sorted(os.listdir(GOLDEN)):
        if not os.path.isdir(os.path.join(GOLDEN, d)):
            continue
        k = json.load(open(os.path.join(GOLDEN, d, "meta.json"))).get("kind", "graph")
        if k == kind:
            out.append(d)
    return out


def generate(spec):
    name, kw = spec
    return getattr(synthetic, name)(**kw)


def materialize(name: str, root: str):
    """Writes the index of fixture `name` under root/name; returns (path, meta, queries, golden).
    For a QBG fixture the path is the QBG index directory (its global index in path/global)."""
    src = os.path.join(GOLDEN, name)
    meta = json.load(open(os.path.join(src, "meta.json")))
    out = os.path.join(root, name)
    if meta.get("kind") == "qbg":
        if not os.path.exists(os.path.join(out, "grp")):
            with tarfile.open(os.path.join(src, "qbg.tar.gz")) as tf:
                for m in tf.getmembers():
                    dst = os.path.join(out, m.name)
                    os.makedirs(os.path.dirname(dst), exist_ok=True)
                    with tf.extractfile(m) as fi, open(dst, "wb") as fo:
                        fo.write(fi.read())
        return out, meta, generate(meta["query"]), np.load(os.path.join(src, "golden.npz"))
    if not os.path.exists(os.path.join(out, "obj")):
        os.makedirs(out, exist_ok=True)
        shutil.copy(os.path.join(src, "prf"), out)
        for fn in ("grp", "tre", "obj", "robj"):
            p = os.path.join(src, fn + ".gz")
            if os.path.exists(p):
                with gzip.open(p) as fi, open(os.path.join(out, fn), "wb") as fo:
                    fo.write(fi.read())
        qgtar = os.path.join(src, "qg.tar.gz")
        if os.path.exists(qgtar):
            with tarfile.open(qgtar) as tf:
                for m in tf.getmembers():
                    dst = os.path.join(out, "qg", m.name)
                    os.makedirs(os.path.dirname(dst), exist_ok=True)
                    with tf.extractfile(m) as fi, open(dst, "wb") as fo:
                        fo.write(fi.read())
        if meta["regenerate_obj"]:
            base = generate(meta["base"])
            rows = {"f": np.float32, "c": np.uint8, "h": np.float16}[meta["otype"]](base)
            oracle.write_objects(os.path.join(out, "obj"), rows)
    queries = generate(meta["query"])
    golden = np.load(os.path.join(src, "golden.npz"))
    return out, meta, queries, golden


def is_integer_fixture(name: str) -> bool:
    return name in INTEGER_FIXTURES
