"""Index construction for the benchmark workloads (outside the search path).

The reference builds its indexes with its CLI (`ngt create`, `ngt
reconstruct-graph`); that CPU build takes far too long for a 1M-object
benchmark set on a fresh GPU host, so the benchmark builds an equivalent index
on the GPU here and writes it in NGT's on-disk format, after which it is opened
and searched through the C ABI exactly like a reference-built index.

Construction (ONNG, lib/NGT/GraphReconstructor.h:645-760 reconstructGraph):
  1. the exact K-nearest-neighbour graph (K = 100, the ANNG creation edge
     count), from L2 distances computed as |x|^2 + |y|^2 - 2 x.y with an fp32
     GEMM (TF32 off): for integer coordinates <= 255 every product and partial
     sum is an integer below 2^24, so the neighbour lists are exact;
  2. outgoing edges: the first `outgoing` neighbours of every node;
  3. incoming edges: node u is added to the list of each of its first
     `incoming` neighbours (reverse edges), duplicates removed, every list
     sorted by (distance, id).
  4. the reference's path adjustment (shortcut reduction), by the library's GPU
     ONNG construction (ngtgpu_build_onng), which also redoes steps 2-3 exactly as
     GraphReconstructor::reconstructGraph does from the k-NN lists written as an ANNG.

Written files: prf, obj (NGT Repository<Object>), grp (Repository<GraphNode>
with the trailing per-node size vector), and no tree: the index is
IndexType Graph, so searches start from seeded random nodes.  Like a
reference ONNG it searches with the dynamic edge size (EdgeSizeForSearch -2:
30 + 10^(20*epsilon) edges per expanded node, NGT's default base and rate).
"""
from __future__ import annotations

import os
import shutil
import time

import numpy as np


def knn_graph(x: np.ndarray, k: int, chunk: int = 2048, log=print):
    """Exact k-NN lists (excluding self) of the rows of x, as 1-based ids and float32 distances."""
    import torch
    dev = torch.device("cuda")
    n = x.shape[0]
    torch.backends.cuda.matmul.allow_tf32 = False
    X = torch.from_numpy(x).to(dev)
    sq = (X * X).sum(1)                                   # integers < 2^24: exact in fp32
    ids = torch.empty((n, k), dtype=torch.int32, device=dev)
    dst = torch.empty((n, k), dtype=torch.float32, device=dev)
    t0 = time.time()
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        g = X[s:e] @ X.T                                   # fp32 GEMM: exact for integer data <= 255
        d2 = sq[s:e, None] + sq[None, :] - 2.0 * g
        d2[torch.arange(e - s, device=dev), torch.arange(s, e, device=dev)] = float("inf")
        v, i = torch.topk(d2, k, dim=1, largest=False, sorted=True)
        ids[s:e] = i.int() + 1
        dst[s:e] = v.clamp_min(0).sqrt()
        del g, d2
    torch.cuda.synchronize()
    log("knn graph: %d x %d in %.1f s" % (n, k, time.time() - t0))
    return ids, dst


def onng_reconstruct(ids, dst, outgoing: int, incoming: int):
    """ONNG edge sets from the k-NN lists: (offsets[nrows+1], edges[E], dists[E]) with row 0 the dummy."""
    import torch
    n, k = ids.shape
    dev = ids.device
    src_out = torch.arange(1, n + 1, device=dev, dtype=torch.int64)[:, None].expand(n, outgoing).reshape(-1)
    dst_out = ids[:, :outgoing].reshape(-1).long()
    d_out = dst[:, :outgoing].reshape(-1)
    # reverse edges: v gets u for each of u's first `incoming` neighbours v
    src_in = ids[:, :incoming].reshape(-1).long()
    dst_in = torch.arange(1, n + 1, device=dev, dtype=torch.int64)[:, None].expand(n, incoming).reshape(-1)
    d_in = dst[:, :incoming].reshape(-1)
    src = torch.cat([src_out, src_in])
    to = torch.cat([dst_out, dst_in])
    dd = torch.cat([d_out, d_in]).contiguous()
    # order by (src, distance, id): stable sort by id, then by (src, distance bits);
    # distances are >= 0 so their IEEE bits order like integers
    dbits = dd.view(torch.int32).long()
    o1 = torch.argsort(to, stable=True)
    o2 = torch.argsort((src[o1] << 32) | dbits[o1], stable=True)
    order = o1[o2]
    src, to, dd = src[order], to[order], dd[order]
    # a pair can appear as an outgoing and as a reverse edge with the same distance:
    # after the sort the copies are adjacent
    keep = torch.ones_like(src, dtype=torch.bool)
    keep[1:] = (src[1:] != src[:-1]) | (to[1:] != to[:-1])
    src, to, dd = src[keep], to[keep], dd[keep]
    deg = torch.bincount(src, minlength=n + 1)
    offsets = torch.zeros(n + 2, dtype=torch.int64, device=dev)
    offsets[1:] = torch.cumsum(deg, 0)
    return offsets[: n + 2].cpu().numpy(), to.int().cpu().numpy(), dd.cpu().numpy()


def write_index(path: str, x: np.ndarray, offsets: np.ndarray, edges: np.ndarray, dists: np.ndarray,
                extra_prf: dict | None = None) -> None:
    """Writes prf / obj / grp of a float32 L2 graph-only NGT index."""
    os.makedirs(path, exist_ok=True)
    n, dim = x.shape
    nrows = n + 1
    prf = {"Dimension": str(dim), "DistanceType": "L2", "ObjectType": "Float-4", "IndexType": "Graph",
           "GraphType": "ONNG", "EdgeSizeForSearch": "-2", "EdgeSizeForCreation": "100", "SeedSize": "10",
           "SeedType": "None", "EpsilonType": "None", "DynamicEdgeSizeBase": "30", "DynamicEdgeSizeRate": "20",
           "DatabaseType": "Memory", "ObjectAlignment": "False", "RefinementObjectType": "Float-4",
           "OutgoingEdge": "10", "IncomingEdge": "100"}
    prf.update(extra_prf or {})
    with open(os.path.join(path, "prf"), "w") as f:
        for kk in sorted(prf):
            f.write("%s\t%s\n" % (kk, prf[kk]))
    # obj
    raw = np.ascontiguousarray(x, np.float32).view(np.uint8).reshape(n, -1)
    rec = np.empty((n, 1 + raw.shape[1]), np.uint8)
    rec[:, 0] = ord("+")
    rec[:, 1:] = raw
    with open(os.path.join(path, "obj"), "wb") as f:
        f.write(np.uint64(nrows).tobytes())
        f.write(b"-")
        f.write(rec.tobytes())
    # grp: per node '+', uint32 count, count x (uint32 id, float32 distance); then uint32 n + uint16[n]
    offsets = np.asarray(offsets, np.int64)
    deg = np.diff(offsets)                                       # nrows entries (row 0 = 0)
    pairs = np.empty((len(edges), 2), np.uint32)
    pairs[:, 0] = edges
    pairs[:, 1] = np.asarray(dists, np.float32).view(np.uint32)
    with open(os.path.join(path, "grp"), "wb") as f:
        f.write(np.uint64(nrows).tobytes())
        f.write(b"-")
        step = 8192
        for a in range(1, nrows, step):
            b = min(nrows, a + step)
            d = deg[a:b]
            sizes = 5 + 8 * d
            starts = np.concatenate([[0], np.cumsum(sizes)[:-1]])
            buf = np.empty(int(sizes.sum()), np.uint8)
            buf[starts] = ord("+")
            cb = d.astype(np.uint32).view(np.uint8).reshape(-1, 4)
            for t in range(4):
                buf[starts + 1 + t] = cb[:, t]
            e0, e1 = offsets[a], offsets[b]
            pb = pairs[e0:e1].view(np.uint8).reshape(-1)
            node = np.repeat(np.arange(b - a), d)
            rank = np.arange(e1 - e0) - (offsets[a:b][node] - e0)
            base = starts[node] + 5 + 8 * rank
            for t in range(8):
                buf[base + t] = pb[t::8]
            f.write(buf.tobytes())
        f.write(np.uint32(nrows).tobytes())
        f.write(np.zeros(nrows, np.uint16).tobytes())


def build_onng_index(path: str, x: np.ndarray, k: int = 100, outgoing: int = 10, incoming: int = 100, log=print,
                     path_adjustment: bool = True):
    """path_adjustment: the k-NN lists are written as an ANNG and turned into an ONNG
    by the library's GPU construction (ngtgpu_build_onng: the reference's graph
    reconstruction and path adjustment, `ngt reconstruct-graph -m S -o outgoing -i
    incoming`); otherwise only the reconstruction, without path adjustment, here."""
    t0 = time.time()
    ids, dst = knn_graph(x, k, log=log)
    if path_adjustment:
        from .base import build_onng
        n = ids.shape[0]
        offsets = np.zeros(n + 2, np.int64)
        offsets[2:] = np.cumsum(np.full(n, k, np.int64))
        anng = path + "_anng"
        if os.path.exists(anng):
            shutil.rmtree(anng)
        write_index(anng, x, offsets, ids.cpu().numpy().reshape(-1), dst.cpu().numpy().reshape(-1),
                    extra_prf={"GraphType": "ANNG"})
        if os.path.exists(path):
            shutil.rmtree(path)
        t1 = time.time()
        build_onng(anng, path, outgoing, incoming, 0)
        shutil.rmtree(anng)
        log("onng construction (GPU path adjustment) in %.1f s" % (time.time() - t1))
    else:
        offsets, edges, dists = onng_reconstruct(ids, dst, outgoing, incoming)
        deg = np.diff(offsets)[1:]
        log("onng reconstruction: %d edges, mean degree %.1f, max %d" % (len(edges), deg.mean(), deg.max()))
        write_index(path, x, offsets, edges, dists)
    log("index written to %s in %.1f s total" % (path, time.time() - t0))
    return ids


def quantize_symmetric(x: np.ndarray, scale: float) -> np.ndarray:
    """int8 codes of NGT's scalar quantization (ObjectSpace::quantizeSymmetrically,
    lib/NGT/ObjectSpace.h:432-441): the division in float32, the product with 127.5
    and the rounding (half away from zero) in float64, clamped to [-127, 127]."""
    v = (np.asarray(x, np.float32) / np.float32(scale)).astype(np.float64) * 127.5
    r = np.sign(v) * np.floor(np.abs(v) + 0.5)
    return np.clip(r, -127, 127).astype(np.int8)


def write_qsint8_index(path: str, float_index: str, x: np.ndarray, log=print) -> float:
    """A QSUInteger-8B (scalar-quantized, L2) graph-only index at `path` over the
    objects x, with the graph of the float index at `float_index`.  The scale is
    max(|max|, |min|) of the objects (NGT::Index::setQuantizationFromMaxMin,
    lib/NGT/Index.cpp:864-875, clipping rate 0).  Returns the scale."""
    t0 = time.time()
    os.makedirs(path, exist_ok=True)
    scale = float(max(abs(float(x.max())), abs(float(x.min()))))
    n, dim = x.shape
    with open(os.path.join(float_index, "prf")) as f:
        prf = dict(line.rstrip("\n").split("\t", 1) for line in f if "\t" in line)
    prf.update({"ObjectType": "QSUInteger-8B", "QuantizationScale": "%.9g" % scale, "QuantizationOffset": "0",
                "QuantizationClippingRate": "0"})
    with open(os.path.join(path, "prf"), "w") as f:
        for kk in sorted(prf):
            f.write("%s\t%s\n" % (kk, prf[kk]))
    rec = np.empty((n, 1 + dim), np.uint8)
    rec[:, 0] = ord("+")
    for a in range(0, n, 1 << 18):
        rec[a:a + (1 << 18), 1:] = quantize_symmetric(x[a:a + (1 << 18)], scale).view(np.uint8)
    with open(os.path.join(path, "obj"), "wb") as f:
        f.write(np.uint64(n + 1).tobytes())
        f.write(b"-")
        f.write(rec.tobytes())
    shutil.copyfile(os.path.join(float_index, "grp"), os.path.join(path, "grp"))
    log("qsint8 index written to %s in %.1f s (scale %g)" % (path, time.time() - t0, scale))
    return scale

