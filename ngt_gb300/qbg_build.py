"""Quantized-blob-graph (QBG) construction for the benchmark workloads (outside the
search path).

The reference builds a QBG index with `qbg create` + `qbg append` + `qbg build`
(hierarchical k-means, its optimizer, CPU); that tool does not exist on a GPU host
without the reference sources, so the benchmark writes one here, on the GPU, in the
reference's on-disk format, and opens it through `qbg_open_index` like a
reference-built index:

  prf          Dimension, GenuineDimension, LocalDivisionNo (subspaces), 16 local
               centroids, GenuineDataType 0 (uint8 objects)
  qr           uint32 dim*dim, then the rotation R, element [p * dim + c]
               (a query x is rotated to x R; lib/NGT/NGTQ/Quantizer.h:117-160)
  rqcb         uint32 (centroids * dim, dim, dim), then the rotated centroids of the
               blob subspace ids ("global codebook")
  local-i/obj  the 16 centroids of subspace i (an NGT object file of dsv floats)
  grp          uint64 subspaces, uint64 nodes (blobs + 1), then per node: uint32
               subspace id, uint32 count, the object ids, and their 4-bit codes in
               16-object blocks of 8 bytes per subspace (object o's code in byte
               8 s + (o % 16) / 2 of its block, low nibble for even o;
               QuantizedObjectProcessingStream, lib/NGT/NGTQ/Quantizer.h:1040-1180)
  global/      an NGT index (prf, obj, grp) over the blob centroids, unrotated: a
               graph-only ONNG (no tree, so searches start from fixed random seeds)
  obj          the object list, an array file (lib/NGT/ArrayFile.h): 16-byte head
               (record size, reserved), per object a 16-byte flag block and the
               object; record 0 unused

Quantizer: blobs from k-means of the objects (Lloyd iterations on a sample, then
every object assigned to its nearest blob), subspace ids from k-means of the blob
centroids, a random orthogonal rotation (QR of a Gaussian matrix), and 16
centroids per dsv-dimensional subspace from k-means of the rotated residuals
(object x R minus the rotated centroid of its blob's subspace id).
"""
from __future__ import annotations

import os
import struct
import time

import numpy as np

from .graph_build import build_onng_index
from .qg_build import write_object_file


def _kmeans(X, k: int, iters: int, seed: int, chunk: int = 16384):
    """Lloyd's k-means of the rows of the GPU tensor X (float32): centroids [k, d]."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    C = X[torch.randperm(X.shape[0], generator=g)[:k].to(X.device)].clone()
    for _ in range(iters):
        a = _assign(X, C, chunk)
        S = torch.zeros_like(C).index_add_(0, a, X)
        cnt = torch.zeros(k, device=X.device).index_add_(0, a, torch.ones_like(a, dtype=torch.float32))
        upd = cnt > 0
        C[upd] = S[upd] / cnt[upd][:, None]
    return C


def _assign(X, C, chunk: int = 16384):
    """Index of the nearest centroid of every row of X."""
    import torch
    cn = (C * C).sum(1)
    out = torch.empty(X.shape[0], dtype=torch.int64, device=X.device)
    for s in range(0, X.shape[0], chunk):
        x = X[s:s + chunk]
        out[s:s + chunk] = (cn[None, :] - 2.0 * (x @ C.T)).argmin(1)
    return out


def build_qbg(path: str, x: np.ndarray, nblobs: int = 65536, nsid: int = 1024, dsv: int = 2, sample: int = 2_000_000,
              iters: int = 10, seed: int = 41, log=print) -> None:
    """Writes a QBG index over the uint8 objects x (ids 1..n) at `path`."""
    import torch
    t0 = time.time()
    dev = torch.device("cuda")
    n, d = x.shape
    if d % dsv or d % 16:
        raise ValueError("dimension must be a multiple of 16 and of the subvector dimension")
    m = d // dsv
    ma = (m + 1) // 2 * 2
    os.makedirs(path, exist_ok=True)
    tf32 = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True          # clustering only: assignments may round
    try:
        X = torch.from_numpy(np.ascontiguousarray(x)).to(dev).float()
        rng = np.random.default_rng(seed)
        pick = torch.from_numpy(rng.choice(n, size=min(sample, n), replace=False)).to(dev)
        B = _kmeans(X[pick], nblobs, iters, seed)
        blob = _assign(X, B)
        cnt = torch.bincount(blob, minlength=nblobs)
        S = torch.zeros_like(B).index_add_(0, blob, X)
        B[cnt > 0] = S[cnt > 0] / cnt[cnt > 0][:, None].float()
        log("qbg: %d blobs (sizes %d..%d) in %.1f s" % (nblobs, int(cnt.min()), int(cnt.max()), time.time() - t0))
        G = _kmeans(B, nsid, iters * 2, seed + 1)
        sid = _assign(B, G)
        Q, _ = torch.linalg.qr(torch.from_numpy(rng.standard_normal((d, d))).to(dev))
        R = Q.float().contiguous()                          # y = x R
        GR = G @ R                                          # rotated subspace-id centroids
        # local codebooks from rotated residuals of a sample
        sub = pick[:min(1_000_000, len(pick))]
        res = (X[sub] @ R - GR[sid[blob[sub]]]).view(-1, m, dsv).transpose(0, 1).contiguous()      # m, S, dsv
        L = res[:, torch.from_numpy(rng.choice(res.shape[1], 16, replace=False)).to(dev), :].clone()  # m, 16, dsv
        for _ in range(20):
            a = torch.cdist(res, L).argmin(2)
            Ssum = torch.zeros_like(L).scatter_add_(1, a[..., None].expand(-1, -1, dsv), res)
            c = torch.zeros(L.shape[:2], device=dev).scatter_add_(1, a, torch.ones_like(a, dtype=torch.float32))
            upd = c > 0
            L[upd] = Ssum[upd] / c[upd][:, None]
        del res
        codes = np.zeros((n, ma), np.uint8)
        for s in range(0, n, 1 << 18):
            r = (X[s:s + (1 << 18)] @ R - GR[sid[blob[s:s + (1 << 18)]]]).view(-1, m, dsv).transpose(0, 1)
            codes[s:s + (1 << 18), :m] = torch.cdist(r, L).argmin(2).transpose(0, 1).to(torch.uint8).cpu().numpy()
        log("qbg: quantizer trained, %d objects encoded in %.1f s" % (n, time.time() - t0))
        blob_np = blob.cpu().numpy()
        sid_np = sid.cpu().numpy().astype(np.uint32)
        B_np = B.cpu().numpy().astype(np.float32)
        R_np = R.cpu().numpy()
        GR_np = GR.cpu().numpy().astype(np.float32)
        L_np = L.cpu().numpy().astype(np.float32)
        del X
    finally:
        torch.backends.cuda.matmul.allow_tf32 = tf32
    # global index over the blob centroids (ids 1..nblobs, node b = blob b - 1)
    build_onng_index(os.path.join(path, "global"), B_np, k=min(100, nblobs - 1), outgoing=10, incoming=100, log=log,
                     path_adjustment=False)
    # blobs: members in id order
    order = np.argsort(blob_np, kind="stable")
    counts = np.bincount(blob_np, minlength=nblobs)
    starts = np.concatenate([[0], np.cumsum(counts)])
    with open(os.path.join(path, "grp"), "wb", buffering=1 << 24) as f:
        f.write(np.array([m, nblobs + 1], np.uint64).tobytes())
        f.write(struct.pack("<II", 0, 0))                   # node 0: the unused slot
        for b in range(nblobs):
            members = order[starts[b]:starts[b + 1]]
            k = len(members)
            f.write(struct.pack("<II", int(sid_np[b]), k))
            if k:
                f.write((members + 1).astype(np.uint32).tobytes())
                nblk = (k + 15) // 16
                c = np.zeros((nblk * 16, ma), np.uint8)
                c[:k] = codes[members]
                c = c.reshape(nblk, 16, ma).transpose(0, 2, 1)          # blocks, subspaces, objects
                f.write((c[:, :, 0::2] | (c[:, :, 1::2] << 4)).astype(np.uint8).tobytes())
    with open(os.path.join(path, "qr"), "wb") as f:
        f.write(np.uint32(d * d).tobytes())
        f.write(np.ascontiguousarray(R_np, np.float32).tobytes())
    with open(os.path.join(path, "rqcb"), "wb") as f:
        f.write(np.array([nsid * d, d, d], np.uint32).tobytes())
        f.write(GR_np.tobytes())
    for s in range(m):
        os.makedirs(os.path.join(path, "local-%d" % s), exist_ok=True)
        write_object_file(os.path.join(path, "local-%d" % s, "obj"), L_np[s])
    with open(os.path.join(path, "prf"), "w") as f:
        for kv in (("Dimension", d), ("GenuineDimension", d), ("LocalDivisionNo", m), ("LocalCentroidLimit", 16),
                   ("GlobalCentroidLimit", nsid), ("SingleLocalCodebook", 0), ("DistanceType", 1),
                   ("DataType", 1), ("GenuineDataType", 0), ("QuantizerType", 2)):
            f.write("%s\t%s\n" % kv)
    # the object list
    with open(os.path.join(path, "obj"), "wb", buffering=1 << 24) as f:
        f.write(np.array([d, 0], np.uint64).tobytes())
        f.write(np.zeros(16 + d, np.uint8).tobytes())
        for s in range(0, n, 1 << 20):
            rows = x[s:s + (1 << 20)]
            rec = np.zeros((rows.shape[0], 16 + d), np.uint8)
            rec[:, 16:] = rows
            f.write(rec.tobytes())
    log("qbg: index written to %s in %.1f s" % (path, time.time() - t0))
