"""Quantized-graph construction for the benchmark workloads (outside the search path).

The reference quantizes an index with `qbg create-qg` + `qbg build-qg` (CPU,
with its own optimizer); that tool does not exist on a GPU host without the
reference sources, so the benchmark writes a quantized graph here, in the
reference's on-disk format (lib/NGT/NGTQ/QuantizedGraph.h:167-229 for grp,
lib/NGT/NGTQ/Quantizer.h for prf / qr / rqcb / local-*), and then opens it
through `ngtqg_open_index` like a reference-built one.

Quantizer: no rotation (an empty qr), a zero global centroid, and 16 centroids
per `dsv`-dimensional subspace from k-means (20 Lloyd iterations on a sample,
on the GPU).  Every node keeps its first `max_edges` graph edges and the 4-bit
codes of those neighbours: blocks of 16 neighbours, per subspace 8 bytes,
neighbour o's code in byte 8*s + o/2 of its block, low nibble for even o
(QuantizedObjectProcessingStream, lib/NGT/NGTQ/Quantizer.h:1040-1180).
"""
from __future__ import annotations

import os
import struct
import time

import numpy as np


def read_graph(index_path: str):
    """CSR of an NGT grp file (Repository<GraphNode>: per slot '-' or '+', uint32 count,
    count x (uint32 id, float distance)): offsets[n+1], edges (uint32), row 0 the dummy."""
    buf = open(os.path.join(index_path, "grp"), "rb").read()
    n = struct.unpack_from("<Q", buf, 0)[0]
    pos = 8
    counts = np.zeros(n, np.int64)
    lists = []
    for i in range(n):
        if buf[pos] == ord("-"):
            pos += 1
            continue
        c = struct.unpack_from("<I", buf, pos + 1)[0]
        counts[i] = c
        lists.append(np.frombuffer(buf, np.uint32, 2 * c, pos + 5)[::2])
        pos += 5 + 8 * c
    offsets = np.zeros(n + 1, np.int64)
    offsets[1:] = np.cumsum(counts)
    edges = np.concatenate(lists).astype(np.uint32) if lists else np.zeros(0, np.uint32)
    return offsets, edges


def train_pq(x: np.ndarray, dsv: int, sample: int = 65536, iters: int = 20, seed: int = 0):
    """16 centroids per subspace: returns float32 [m][16][dsv]."""
    import torch
    dev = torch.device("cuda")
    rng = np.random.default_rng(seed)
    n, d = x.shape
    m = d // dsv
    pick = rng.choice(n, size=min(sample, n), replace=False)
    X = torch.from_numpy(np.ascontiguousarray(x[pick], np.float32)).to(dev).view(-1, m, dsv).transpose(0, 1)  # m,S,dsv
    C = X[:, torch.from_numpy(rng.choice(X.shape[1], 16, replace=False)).to(dev), :].clone()                # m,16,dsv
    for _ in range(iters):
        d2 = torch.cdist(X, C) ** 2                                     # m,S,16
        a = d2.argmin(2)                                                # m,S
        S = torch.zeros_like(C).scatter_add_(1, a[..., None].expand(-1, -1, dsv), X)
        cnt = torch.zeros(C.shape[:2], device=dev).scatter_add_(1, a, torch.ones_like(a, dtype=torch.float32))
        upd = cnt > 0
        C[upd] = S[upd] / cnt[upd][:, None]
    return C.cpu().numpy()


def encode(x: np.ndarray, C: np.ndarray, chunk: int = 65536):
    """4-bit codes [n][m] (uint8 values 0..15): nearest centroid per subspace."""
    import torch
    dev = torch.device("cuda")
    m, _, dsv = C.shape
    Ct = torch.from_numpy(C).to(dev)
    out = np.zeros((x.shape[0], m), np.uint8)
    for s in range(0, x.shape[0], chunk):
        X = torch.from_numpy(np.ascontiguousarray(x[s:s + chunk], np.float32)).to(dev).view(-1, m, dsv).transpose(0, 1)
        out[s:s + chunk] = (torch.cdist(X, Ct) ** 2).argmin(2).transpose(0, 1).to(torch.uint8).cpu().numpy()
    return out


def write_object_file(path: str, rows: np.ndarray) -> None:
    rows = np.ascontiguousarray(rows, np.float32)
    rec = np.empty((rows.shape[0], 1 + rows.shape[1] * 4), np.uint8)
    rec[:, 0] = ord("+")
    rec[:, 1:] = rows.view(np.uint8).reshape(rows.shape[0], -1)
    with open(path, "wb") as f:
        f.write(np.uint64(rows.shape[0] + 1).tobytes())
        f.write(b"-")
        f.write(rec.tobytes())


def build_qg(index_path: str, x: np.ndarray, dsv: int = 2, max_edges: int = 128, log=print) -> None:
    """Writes index_path/qg for the NGT index at index_path whose objects (ids 1..n) are x."""
    t0 = time.time()
    n, d = x.shape
    if d % dsv:
        raise ValueError("dimension not a multiple of the subvector dimension")
    m = d // dsv
    ma = (m + 1) // 2 * 2
    qg = os.path.join(index_path, "qg")
    os.makedirs(qg, exist_ok=True)
    offsets, edges = read_graph(index_path)
    C = train_pq(x, dsv)
    codes = np.zeros((n + 1, ma), np.uint8)                    # row 0: the dummy object
    codes[1:, :m] = encode(x, C)
    log("qg: quantizer trained and %d objects encoded in %.1f s" % (n, time.time() - t0))
    # grp: uint64 subspaces, uint64 nodes, then per node: subspace id 0, count, its first
    # max_edges edge ids, and their codes in 16-neighbour blocks (padding slots: code 0)
    nn = len(offsets) - 1
    cnt_all = np.minimum(np.diff(offsets), max_edges).astype(np.int64)
    total_bytes = 0
    with open(os.path.join(qg, "grp"), "wb", buffering=1 << 24) as f:
        f.write(np.array([m, nn], np.uint64).tobytes())
        for a in range(0, nn, 65536):
            b = min(nn, a + 65536)
            cnt = cnt_all[a:b]
            nblk = (cnt + 15) // 16
            slot0 = np.zeros(len(cnt) + 1, np.int64)
            slot0[1:] = np.cumsum(nblk * 16)
            nbr = np.zeros(slot0[-1], np.int64)
            node = np.repeat(np.arange(len(cnt)), cnt)
            within = np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt)
            nbr[slot0[node] + within] = edges[offsets[a + node] + within]
            c = codes[nbr].reshape(-1, 16, ma).transpose(0, 2, 1)         # blocks, subspaces, neighbours
            packed = (c[:, :, 0::2] | (c[:, :, 1::2] << 4)).astype(np.uint8).reshape(-1)
            for i in range(len(cnt)):
                k = int(cnt[i])
                f.write(struct.pack("<II", 0, k))
                if k:
                    e0 = offsets[a + i]
                    f.write(edges[e0:e0 + k].astype(np.uint32).tobytes())
                    s0 = slot0[i] * ma // 2
                    f.write(packed[s0:s0 + nblk[i] * 8 * ma].tobytes())
                    total_bytes += int(nblk[i] * 8 * ma)
    with open(os.path.join(qg, "qr"), "wb") as f:
        f.write(np.uint32(0).tobytes())
    with open(os.path.join(qg, "rqcb"), "wb") as f:
        f.write(np.array([d, d, d], np.uint32).tobytes())
        f.write(np.zeros(d, np.float32).tobytes())
    for s in range(m):
        os.makedirs(os.path.join(qg, "local-%d" % s), exist_ok=True)
        write_object_file(os.path.join(qg, "local-%d" % s, "obj"), C[s])
    with open(os.path.join(qg, "prf"), "w") as f:
        for kv in (("Dimension", d), ("GenuineDimension", d), ("LocalDivisionNo", m), ("LocalCentroidLimit", 16),
                   ("GlobalCentroidLimit", 1), ("SingleLocalCodebook", 0), ("DistanceType", 1), ("DataType", 1)):
            f.write("%s\t%s\n" % kv)
    log("qg: written to %s in %.1f s (%.2f GB of codes)" % (qg, time.time() - t0, total_bytes / 1e9))
