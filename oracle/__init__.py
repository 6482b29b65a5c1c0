"""ORACLE -- test infrastructure only.

Python side of the CPU restatement of NGT's search path (ngt_oracle.c):
an independent numpy reader of the NGT index directory and a ctypes binding
of the C restatement.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline use it, always as the checker or the timed CPU reference; the
product (ngt_gb300/) never imports it.

Index file formats restated from the reference:
  prf  text key/value           lib/NGT/Common.h:915-1000
  obj  Repository<Object>       lib/NGT/Common.h:2181-2238, lib/NGT/ObjectSpace.h:620-640
  grp  Repository<GraphNode>    lib/NGT/Graph.h:153-160, lib/NGT/ObjectSpace.h:72-80
  tre  DVP tree                 lib/NGT/Tree.h:347-355, lib/NGT/Node.h:88-110,218-280,441-510

Quantized-graph files (<index>/qg, written by `qbg create-qg` / `qbg build-qg`):
  prf       text key/value (NGTQ::Property)      lib/NGT/NGTQ/Quantizer.h:560-700
  qr        uint32 n, n floats (Rotation)        lib/NGT/NGTQ/Quantizer.h:164-186
  rqcb      uint32 size, dimension, paddedDimension, floats (QuantizationCodebook)
                                                 lib/NGT/NGTQ/Quantizer.h:355-378
  local-i   NGT index whose obj holds subspace i's 16 centroids
  grp       uint64 subspaces, uint64 n, per node uint32 sid, uint32 count, count ids,
            the node's 4-bit code stream          lib/NGT/NGTQ/QuantizedGraph.h:170-226
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
FAST_LIB_PATH = os.path.join(HERE, "_build", "liboracle_fast.so")

OBJTYPES = {"Float-4": 0, "Integer-1": 1, "Float-2": 2, "QSUInteger-8B": 3}
ELEM = {0: np.float32, 1: np.uint8, 2: np.float16, 3: np.int8}
METRICS = {"L1": 0, "L2": 1, "Hamming": 2, "Angle": 3, "Cosine": 4, "NormalizedAngle": 5,
           "NormalizedCosine": 6, "Jaccard": 7, "NormalizedL2": 9, "InnerProduct": 10,
           "Poincare": 100, "Lorentz": 101}


def build(verbose: bool = False) -> str:
    """Compiles liboracle.so (gcc, OpenMP) when it is missing or stale."""
    src = os.path.join(HERE, "ngt_oracle.c")
    if os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src):
        return LIB_PATH
    r = subprocess.run(["make", "-C", HERE, "port"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    if verbose:
        print(r.stdout)
    return LIB_PATH


def epsilon_from_accuracy(table: str, accuracy: float) -> float:
    """AccuracyTable::getEpsilon (lib/NGT/Index.h:442-472): epsilon interpolated
    between the two table entries around the expected accuracy (float epsilons, double
    accuracies, the difference of the epsilons in float)."""
    t = []
    for tok in table.split(","):
        if not tok:
            continue
        a, b = tok.split(":")
        t.append((np.float32(float(a)), float(b)))
    if len(t) <= 2:
        raise ValueError("the accuracy table is not set")
    accuracy = min(accuracy, 1.0)
    i = 0
    while i < len(t) and t[i][1] < accuracy:
        i += 1
    if i == len(t):
        i -= 2
    elif i != 0:
        i -= 1
    lo, up = t[i], t[i + 1]
    e = np.float32(float(lo[0]) + float(np.float32(up[0] - lo[0])) * (accuracy - lo[1]) / (up[1] - lo[1]))
    return float(max(e, np.float32(-0.9)))


def build_fast() -> str:
    """Compiles liboracle_fast.so: the same restatement with the reference's Release
    flags (-Ofast -march=native), timed as the CPU baseline; never used to check."""
    src = os.path.join(HERE, "ngt_oracle.c")
    if os.path.exists(FAST_LIB_PATH) and os.path.getmtime(FAST_LIB_PATH) >= os.path.getmtime(src):
        return FAST_LIB_PATH
    r = subprocess.run(["make", "-C", HERE, "fast"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle speed build failed:\n" + r.stdout + r.stderr)
    return FAST_LIB_PATH


class OracleIndexC(ctypes.Structure):
    _fields_ = [("otype", ctypes.c_int), ("metric", ctypes.c_int),
                ("nrows", ctypes.c_uint32), ("dpad", ctypes.c_uint32),
                ("objects", ctypes.c_void_p), ("present", ctypes.c_void_p),
                ("offsets", ctypes.c_void_p), ("edges", ctypes.c_void_p),
                ("has_tree", ctypes.c_int),
                ("root", ctypes.c_uint32), ("ninternals", ctypes.c_uint32), ("nleaves", ctypes.c_uint32),
                ("in_pivot", ctypes.c_void_p), ("in_nchildren", ctypes.c_void_p), ("in_children", ctypes.c_void_p),
                ("in_borders", ctypes.c_void_p), ("pivots", ctypes.c_void_p),
                ("leaf_first", ctypes.c_void_p), ("leaf_count", ctypes.c_void_p), ("leaf_ids", ctypes.c_void_p),
                ("seed_size", ctypes.c_int), ("seed_type", ctypes.c_int), ("epsilon_type", ctypes.c_int),
                ("edge_size_for_search", ctypes.c_int), ("dyn_base", ctypes.c_int), ("dyn_rate", ctypes.c_int)]


def read_property(path: str) -> dict:
    prop = {}
    with open(os.path.join(path, "prf")) as f:
        for line in f:
            line = line.rstrip("\r\n")
            if "\t" in line:
                k, v = line.split("\t", 1)
                prop[k] = v
    return prop


class IndexFiles:
    """numpy view of an NGT index directory (object rows padded to 16 elements)."""

    def __init__(self, path: str):
        self.path = path
        self.prop = read_property(path)
        self.dimension = int(self.prop["Dimension"])
        self.metric_name = self.prop.get("DistanceType", "L2")
        self.metric = METRICS[self.metric_name]
        self.otype = OBJTYPES[self.prop.get("ObjectType", "Float-4")]
        self.dtype = ELEM[self.otype]
        self.dim = self.dimension + (1 if self.metric_name == "InnerProduct" else 0)
        self.dpad = ((self.dim - 1) // 16 + 1) * 16
        self.has_tree = self.prop.get("IndexType", "GraphAndTree") == "GraphAndTree"
        self._read_obj()
        self._read_grp()
        if self.has_tree:
            self._read_tre()

    def refinement_objects(self):
        """The float refinement objects (robj) of the index, or None: rows of the user
        dimension, slot 0 unused (lib/NGT/Index.cpp:1207)."""
        p = os.path.join(self.path, "robj")
        if not os.path.exists(p) or os.path.getsize(p) <= 8:
            return None
        return _read_rows(p, self.dimension)

    def _read_obj(self):
        buf = open(os.path.join(self.path, "obj"), "rb").read()
        n = int(np.frombuffer(buf, np.uint64, 1, 0)[0])
        es = np.dtype(self.dtype).itemsize
        rowb = self.dim * es
        self.nrows = n
        self.objects = np.zeros((n, self.dpad), self.dtype)
        self.present = np.zeros(n, np.uint8)
        if len(buf) == 9 + (n - 1) * (1 + rowb) and buf[8:9] == b"-":
            # common case: only the dummy slot is empty -> fixed-size records
            rec = np.frombuffer(buf, np.uint8, (n - 1) * (1 + rowb), 9).reshape(n - 1, 1 + rowb)
            if (rec[:, 0] == ord("+")).all():
                self.objects[1:, :self.dim] = np.ascontiguousarray(rec[:, 1:]).view(self.dtype)
                self.present[1:] = 1
                return
        pos = 8
        for i in range(n):
            t = buf[pos:pos + 1]
            pos += 1
            if t == b"-":
                continue
            assert t == b"+", "corrupted object file"
            self.objects[i, :self.dim] = np.frombuffer(buf, self.dtype, self.dim, pos)
            self.present[i] = 1
            pos += rowb
        assert pos == len(buf), "trailing bytes in the object file"

    def _read_grp(self):
        buf = open(os.path.join(self.path, "grp"), "rb").read()
        lib = ctypes.CDLL(build())
        lib.oracle_parse_graph.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_void_p,
                                           ctypes.c_void_p]
        lib.oracle_parse_graph.restype = ctypes.c_int64
        total = lib.oracle_parse_graph(buf, len(buf), self.nrows, None, None)
        assert total >= 0, "corrupted graph file"
        self.offsets = np.zeros(self.nrows + 1, np.uint32)
        self.edges = np.zeros(max(total, 1), np.uint32)
        lib.oracle_parse_graph(buf, len(buf), self.nrows, self.offsets.ctypes.data, self.edges.ctypes.data)
        self.edges = self.edges[:total]

    def _read_grp_python(self):
        buf = open(os.path.join(self.path, "grp"), "rb").read()
        n = int(np.frombuffer(buf, np.uint64, 1, 0)[0])
        pos = 8
        adj = [np.zeros(0, np.uint32)] * self.nrows
        for i in range(n):
            t = buf[pos:pos + 1]
            pos += 1
            if t == b"-":
                continue
            cnt = int(np.frombuffer(buf, np.uint32, 1, pos)[0])
            pos += 4
            rec = np.frombuffer(buf, np.uint32, 2 * cnt, pos).reshape(cnt, 2)
            adj[i] = rec[:, 0].copy()
            pos += 8 * cnt
        self.offsets = np.zeros(self.nrows + 1, np.uint32)
        self.offsets[1:] = np.cumsum([len(a) for a in adj])
        self.edges = np.concatenate(adj).astype(np.uint32) if self.nrows else np.zeros(0, np.uint32)

    def _read_tre(self):
        buf = open(os.path.join(self.path, "tre"), "rb").read()
        es = np.dtype(self.dtype).itemsize
        rowb = self.dim * es
        pos = 0
        nl = int(np.frombuffer(buf, np.uint64, 1, pos)[0]); pos += 8
        self.leaf_first = np.zeros(nl, np.uint32)
        self.leaf_count = np.zeros(nl, np.uint32)
        ids = []
        for i in range(nl):
            t = buf[pos:pos + 1]; pos += 1
            if t == b"-":
                continue
            _nid, parent = np.frombuffer(buf, np.uint32, 2, pos); pos += 8
            cnt = int(np.frombuffer(buf, np.uint16, 1, pos)[0]); pos += 2
            rec = np.frombuffer(buf, np.uint32, 2 * cnt, pos).reshape(cnt, 2); pos += 8 * cnt
            self.leaf_first[i] = len(ids)
            self.leaf_count[i] = cnt
            ids.extend(rec[:, 0].tolist())
            if not ((int(parent) & 0x7fffffff) == 0 and cnt == 0):
                pos += rowb
        self.leaf_ids = np.array(ids, np.uint32)
        ni = int(np.frombuffer(buf, np.uint64, 1, pos)[0]); pos += 8
        self.in_pivot = np.zeros(ni, np.uint32)
        self.in_nchildren = np.zeros(ni, np.uint32)
        self.in_children = np.zeros((ni, 5), np.uint32)
        self.in_borders = np.zeros((ni, 4), np.float32)
        pivots = []
        for i in range(ni):
            t = buf[pos:pos + 1]; pos += 1
            if t == b"-":
                continue
            pos += 8
            row = np.zeros(self.dpad, self.dtype)
            row[:self.dim] = np.frombuffer(buf, self.dtype, self.dim, pos); pos += rowb
            self.in_pivot[i] = len(pivots)
            pivots.append(row)
            cs = int(np.frombuffer(buf, np.uint64, 1, pos)[0]); pos += 8
            self.in_nchildren[i] = cs
            self.in_children[i, :cs] = np.frombuffer(buf, np.uint32, cs, pos); pos += 4 * cs
            self.in_borders[i, :cs - 1] = np.frombuffer(buf, np.float32, cs - 1, pos); pos += 4 * (cs - 1)
        assert pos == len(buf), "trailing bytes in the tree file"
        self.pivots = np.stack(pivots) if pivots else np.zeros((1, self.dpad), self.dtype)
        self.root = 1 if (ni > 1 and self.in_nchildren[1] > 0) else (0x80000000 | 1)


class OracleQGC(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_uint32), ("m", ctypes.c_uint32), ("ld", ctypes.c_uint32), ("ma", ctypes.c_uint32),
                ("rotation", ctypes.c_void_p), ("gcentroid", ctypes.c_void_p), ("lcentroids", ctypes.c_void_p),
                ("nnodes", ctypes.c_uint32), ("offsets", ctypes.c_void_p), ("ids", ctypes.c_void_p),
                ("code_off", ctypes.c_void_p), ("codes", ctypes.c_void_p), ("sid", ctypes.c_void_p),
                ("olist", ctypes.c_void_p), ("olist_dim", ctypes.c_uint32), ("olist_type", ctypes.c_int),
                ("olist_n", ctypes.c_uint32)]


def read_object_list(path: str, dtype) -> np.ndarray:
    """Rows of a QBG object list (qbg_dir/obj): an array file with a 16-byte head
    (record size, reserved) and records of a 16-byte flag block followed by the
    object (lib/NGT/ArrayFile.h); row 0 is the unused slot."""
    raw = np.fromfile(path, np.uint8)
    rs = int(raw[:8].view(np.uint64)[0])
    n = (len(raw) - 16) // (16 + rs)
    assert (len(raw) - 16) % (16 + rs) == 0, "truncated object list " + path
    rec = raw[16:16 + n * (16 + rs)].reshape(n, 16 + rs)[:, 16:]
    return np.ascontiguousarray(rec).view(dtype)


def _read_rows(path: str, dim: int) -> np.ndarray:
    """Float rows of an NGT object file (slot 0 and deleted slots as zeros)."""
    buf = open(path, "rb").read()
    n = int(np.frombuffer(buf, np.uint64, 1, 0)[0])
    rows = np.zeros((n, dim), np.float32)
    pos = 8
    for i in range(n):
        t = buf[pos:pos + 1]
        pos += 1
        if t == b"-":
            continue
        rows[i] = np.frombuffer(buf, np.float32, dim, pos)
        pos += 4 * dim
    assert pos == len(buf), "trailing bytes in " + path
    return rows


class QGFiles:
    """numpy view of the quantized graph of an index (<index>/qg), or, with
    blobs=True, of a QBG index directory (same file formats at its top level,
    one rotated codebook centroid per blob subspace id, blob codes in grp)."""

    def __init__(self, index_path: str, blobs: bool = False):
        qg = index_path if blobs else os.path.join(index_path, "qg")
        self.prop = read_property(qg)
        self.dim = int(self.prop["Dimension"])
        self.m = int(self.prop["LocalDivisionNo"])
        assert self.dim % self.m == 0, "dimension is not a multiple of the subspace count"
        self.ld = self.dim // self.m
        self.ma = (self.m + 1) // 2 * 2
        assert int(self.prop.get("LocalCentroidLimit", "16")) == 16, "QG needs 16 local centroids"
        raw = open(os.path.join(qg, "qr"), "rb").read()
        n = int(np.frombuffer(raw, np.uint32, 1, 0)[0]) if raw else 0
        self.rotation = np.frombuffer(raw, np.float32, n, 4).reshape(self.dim, self.dim).copy() if n else None
        raw = open(os.path.join(qg, "rqcb"), "rb").read()
        size, _cdim, pdim = (int(v) for v in np.frombuffer(raw, np.uint32, 3, 0))
        cb = np.frombuffer(raw, np.float32, size, 12).reshape(size // pdim, pdim)
        self.ncentroids = cb.shape[0]
        self.gcentroid = np.zeros((self.ncentroids, self.dim), np.float32)
        self.gcentroid[:, :min(pdim, self.dim)] = cb[:, :min(pdim, self.dim)]
        self.lcentroids = np.zeros((self.m, 16, self.ld), np.float32)
        for i in range(self.m):
            rows = _read_rows(os.path.join(qg, "local-%d" % i, "obj"), self.ld)
            assert rows.shape[0] == 17, "local codebook %d does not hold 16 centroids" % i
            self.lcentroids[i] = rows[1:17]
        raw = open(os.path.join(qg, "grp"), "rb").read()
        _nsub, nn = np.frombuffer(raw, np.uint64, 2, 0)
        pos = 16
        counts, ids, code_off, chunks, sids = [], [], [], [], []
        total = 0
        for _ in range(int(nn)):
            sid, cnt = (int(v) for v in np.frombuffer(raw, np.uint32, 2, pos))
            sids.append(sid)
            pos += 8
            ids.append(np.frombuffer(raw, np.uint32, cnt, pos))
            pos += 4 * cnt
            ssz = ((cnt + 15) // 16) * 16 * self.ma // 2 if cnt else 0
            code_off.append(total)
            chunks.append(np.frombuffer(raw, np.uint8, ssz, pos))
            pos += ssz
            total += ssz
            counts.append(cnt)
        assert pos == len(raw), "trailing bytes in the quantized graph"
        self.nnodes = int(nn)
        self.offsets = np.zeros(self.nnodes + 1, np.uint32)
        self.offsets[1:] = np.cumsum(counts)
        self.ids = np.concatenate(ids).astype(np.uint32) if ids else np.zeros(0, np.uint32)
        self.code_off = np.array(code_off, np.uint64)
        self.codes = np.concatenate(chunks) if chunks else np.zeros(0, np.uint8)
        self.sid = np.array(sids, np.uint32)
        assert (self.sid < self.ncentroids).all(), "blob subspace id beyond the codebook"
        # QBG: the object list the refinement reads (GenuineDataType 0 uint8, 1 float)
        self.olist = None
        olist = os.path.join(qg, "obj")
        if blobs and os.path.exists(olist):
            gdt = int(self.prop.get("GenuineDataType", "0"))
            self.olist_type = {0: 1, 1: 0}[gdt]          # oracle object types: 1 uint8, 0 float
            self.olist = read_object_list(olist, np.uint8 if gdt == 0 else np.float32)


class Oracle:
    """ctypes binding of ngt_oracle.c over one IndexFiles."""

    def __init__(self, files: IndexFiles, speed_build: bool = False):
        """speed_build: load the -Ofast build (for timing the CPU baseline only)."""
        self.f = files
        self.lib = ctypes.CDLL(build_fast() if speed_build else build())
        L = self.lib
        L.oracle_graph_search.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                          ctypes.c_size_t, ctypes.c_float, ctypes.c_float, ctypes.c_int64, ctypes.c_int,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.oracle_linear_search.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.oracle_prepare_queries.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint32, ctypes.c_void_p,
                                             ctypes.c_size_t, ctypes.c_size_t, ctypes.c_void_p]
        L.oracle_rand_sequence.argtypes = [ctypes.c_uint32, ctypes.c_size_t, ctypes.c_void_p]
        L.oracle_prepare_qsint8.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                            ctypes.c_float, ctypes.c_int, ctypes.c_void_p]
        L.oracle_distance.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
        L.oracle_distance.restype = ctypes.c_float
        L.oracle_qg_search.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                       ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_float,
                                       ctypes.c_float, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_int]
        L.oracle_qbg_search.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                        ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_size_t,
                                        ctypes.c_float, ctypes.c_float, ctypes.c_size_t, ctypes.c_int64,
                                        ctypes.c_int, ctypes.c_size_t,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_int]
        L.oracle_qg_rotate.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_qg_lut.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p]
        L.oracle_qg_scan.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float, ctypes.c_float,
                                     ctypes.c_uint32, ctypes.c_void_p]
        L.oracle_qg_scan.restype = ctypes.c_float
        self.qg = None
        f = files
        self._keep = []

        def p(a):
            a = np.ascontiguousarray(a)
            self._keep.append(a)
            return a.ctypes.data

        s = OracleIndexC()
        s.otype, s.metric, s.nrows, s.dpad = f.otype, f.metric, f.nrows, f.dpad
        s.objects, s.present, s.offsets, s.edges = p(f.objects), p(f.present), p(f.offsets), p(f.edges)
        s.has_tree = int(f.has_tree)
        if f.has_tree:
            s.root, s.ninternals, s.nleaves = f.root, len(f.in_pivot), len(f.leaf_first)
            s.in_pivot, s.in_nchildren = p(f.in_pivot), p(f.in_nchildren)
            s.in_children, s.in_borders, s.pivots = p(f.in_children), p(f.in_borders), p(f.pivots)
            s.leaf_first, s.leaf_count, s.leaf_ids = p(f.leaf_first), p(f.leaf_count), p(f.leaf_ids)
        prop = f.prop
        s.seed_size = int(prop.get("SeedSize", "10"))
        st = prop.get("SeedType", "None")
        s.seed_type = {"RandomNodes": 1, "FixedNodes": 2, "FirstNode": 3, "AllLeafNodes": 4}.get(st, 0)
        s.epsilon_type = {"ByQuery": 1, "ResultSize": 2}.get(prop.get("EpsilonType", "None"), 0)
        s.edge_size_for_search = int(prop.get("EdgeSizeForSearch", "40"))
        s.dyn_base = int(prop.get("DynamicEdgeSizeBase", "30"))
        s.dyn_rate = int(prop.get("DynamicEdgeSizeRate", "20"))
        self.s = s

    def prepare(self, queries: np.ndarray) -> np.ndarray:
        q = np.ascontiguousarray(queries, np.float32)
        rows = np.zeros((q.shape[0], self.f.dpad), self.f.dtype)
        if self.f.otype == 3:
            self.lib.oracle_prepare_qsint8(self.f.dpad, q.ctypes.data, q.shape[0], q.shape[1],
                                           ctypes.c_float(float(self.f.prop["QuantizationScale"])),
                                           1 if self.f.metric_name == "NormalizedCosine" else 0, rows.ctypes.data)
            return rows
        self.lib.oracle_prepare_queries(self.f.otype, self.f.metric, self.f.dpad, q.ctypes.data, q.shape[0],
                                        q.shape[1], rows.ctypes.data)
        return rows

    def search(self, queries, k=10, epsilon=0.1, radius=-1.0, edge_size=-1, mode="read_only", threads=1,
               seeds=None):
        rows = self.prepare(queries)
        nq = rows.shape[0]
        # room for round((1+epsilon)*k) results (updatable search, EpsilonType ResultSize)
        kout = int(np.ceil(k * (1.0 + max(0.0, epsilon)))) + 1
        ids = np.zeros((nq, kout), np.uint32)
        ds = np.zeros((nq, kout), np.float32)
        n = np.zeros(nq, np.uint32)
        dc = np.zeros(nq, np.uint32)
        sl = so = sc = None
        if seeds is not None:
            lst, off, cnt = seeds
            sl, so, sc = (np.ascontiguousarray(lst, np.uint32), np.ascontiguousarray(off, np.uint32),
                          np.ascontiguousarray(cnt, np.uint32))
        self.lib.oracle_graph_search(ctypes.byref(self.s), rows.ctypes.data, nq, k, kout, epsilon, radius, edge_size,
                                     0 if mode == "read_only" else 1, ids.ctypes.data, ds.ctypes.data,
                                     n.ctypes.data, dc.ctypes.data,
                                     sl.ctypes.data if sl is not None else None,
                                     so.ctypes.data if so is not None else None,
                                     sc.ctypes.data if sc is not None else None, threads)
        w = max(k, int(n.max()) if nq else 0, 1)
        return ids[:, :w], ds[:, :w], n, dc

    def search_refined(self, queries, k=10, epsilon=0.1, expansion=2.0, mode="read_only", threads=1):
        """GraphIndex::search(SearchQuery&) with a refinement expansion (lib/NGT/Index.h:
        1146-1236): the search keeps k x expansion results, which are re-ranked by the
        exact L2 distance over the float refinement objects; the k best by (distance, id)."""
        R = self.f.refinement_objects()
        size = int(np.float32(k) * np.float32(expansion))
        ids, ds, n, dc = self.search(queries, k=size, epsilon=epsilon, mode=mode, threads=threads)
        q = np.ascontiguousarray(queries, np.float32)
        nq = q.shape[0]
        out_i = np.zeros((nq, k), np.uint32)
        out_d = np.zeros((nq, k), np.float32)
        out_n = np.zeros(nq, np.uint32)
        for j in range(nq):
            c = ids[j, :n[j]]
            d = np.array([self.lib.oracle_distance(0, 1, q[j].ctypes.data, np.ascontiguousarray(R[i]).ctypes.data,
                                                   R.shape[1]) for i in c], np.float32)
            order = np.lexsort((c, d))[:k]
            out_n[j] = len(order)
            out_i[j, :len(order)] = c[order]
            out_d[j, :len(order)] = d[order]
        return out_i, out_d, out_n

    def _qg(self, blobs_path=None):
        if self.qg is None:
            g = QGFiles(blobs_path, blobs=True) if blobs_path else QGFiles(self.f.path)
            self.qgf = g
            s = OracleQGC()
            s.dim, s.m, s.ld, s.ma, s.nnodes = g.dim, g.m, g.ld, g.ma, g.nnodes
            s.rotation = self._p(g.rotation) if g.rotation is not None else None
            s.gcentroid, s.lcentroids = self._p(g.gcentroid), self._p(g.lcentroids)
            s.offsets, s.ids, s.code_off, s.codes = (self._p(g.offsets), self._p(g.ids), self._p(g.code_off),
                                                     self._p(g.codes))
            s.sid = self._p(g.sid) if blobs_path else None
            if blobs_path and g.olist is not None:
                s.olist, s.olist_dim, s.olist_type, s.olist_n = (self._p(g.olist), g.olist.shape[1], g.olist_type,
                                                                 g.olist.shape[0])
            self.qg = s
        return self.qg

    def _p(self, a):
        a = np.ascontiguousarray(a)
        self._keep.append(a)
        return a.ctypes.data

    def qg_search(self, queries, k=20, epsilon=0.03, result_expansion=3.0, radius=-1.0, threads=1, seeds=None):
        """ngtqg_search_index_float over the quantized graph (defaults of
        ngtqg_initialize_query_parameters, lib/NGT/NGTQ/Capi.cpp:46-51)."""
        qg = self._qg()
        qf = np.ascontiguousarray(queries, np.float32)
        rows = self.prepare(qf)
        nq = rows.shape[0]
        kk = max(k, 1)
        ids = np.zeros((nq, kk), np.uint32)
        ds = np.zeros((nq, kk), np.float32)
        n = np.zeros(nq, np.uint32)
        dc = np.zeros(nq, np.uint32)
        sl = so = sc = None
        if seeds is not None:
            sl, so, sc = (np.ascontiguousarray(a, np.uint32) for a in seeds)
        self.lib.oracle_qg_search(ctypes.byref(self.s), ctypes.byref(qg), qf.ctypes.data, qf.shape[1],
                                  rows.ctypes.data, nq, k, epsilon, result_expansion, radius, ids.ctypes.data,
                                  ds.ctypes.data, n.ctypes.data, dc.ctypes.data,
                                  sl.ctypes.data if sl is not None else None,
                                  so.ctypes.data if so is not None else None,
                                  sc.ctypes.data if sc is not None else None, threads)
        return ids, ds, n, dc

    def qbg_search(self, queries, qbg_path, k=20, epsilon=0.1, blob_epsilon=0.0, result_expansion=3.0,
                   explored_blobs=256, edges=0, threads=1, two_step=False, refinement_expansion=None):
        """qbg_search_index_float over a QBG index whose global index this Oracle
        was built on (defaults of qbg_initialize_query_parameters,
        lib/NGT/NGTQ/Capi.cpp:528-536).  Returns ids, distances, counts, blobs judged.

        two_step: searchInTwoSteps with explored_blobs probes.  refinement_expansion
        (>= 1): the search keeps k x expansion results, re-ranked by exact distance
        over the object list to the k best (the search containers of the reference's
        CLI and ngtpy); it replaces result_expansion."""
        refine = refinement_expansion is not None and refinement_expansion >= 1.0
        if refinement_expansion is not None:
            result_expansion = refinement_expansion
        qg = self._qg(qbg_path)
        qf = np.zeros((len(queries), self.f.dpad), np.float32)
        q = np.asarray(queries, np.float32)
        qf[:, :q.shape[1]] = q
        rows = self.prepare(q)
        nq = rows.shape[0]
        size = int(np.float32(k) * np.float32(result_expansion)) if result_expansion >= 1.0 else k
        kout = max(size, 1)
        ids = np.zeros((nq, kout), np.uint32)
        ds = np.zeros((nq, kout), np.float32)
        n = np.zeros(nq, np.uint32)
        nb = np.zeros(nq, np.uint32)
        if refine and not qg.olist:
            raise ValueError("the refinement needs the QBG object list (qbg_dir/obj)")
        self.lib.oracle_qbg_search(ctypes.byref(self.s), ctypes.byref(qg), qf.ctypes.data, self.f.dpad,
                                   rows.ctypes.data, nq, size, kout, epsilon, blob_epsilon, explored_blobs, edges,
                                   1 if two_step else 0, k if refine else 0,
                                   ids.ctypes.data, ds.ctypes.data, n.ctypes.data, nb.ctypes.data, threads)
        return ids, ds, n, nb

    def qg_lut(self, query):
        """Rotated query, uint8 lookup table, scale and offset of one query."""
        qg = self._qg()
        x = np.zeros(qg.dim, np.float32)
        q = np.asarray(query, np.float32)
        x[:min(len(q), qg.dim)] = q[:qg.dim]
        rq = np.zeros(qg.dim, np.float32)
        self.lib.oracle_qg_rotate(ctypes.byref(qg), x.ctypes.data, rq.ctypes.data)
        lut = np.zeros(qg.m * 16, np.uint8)
        sc, of = ctypes.c_float(), ctypes.c_float()
        self.lib.oracle_qg_lut(ctypes.byref(qg), rq.ctypes.data, lut.ctypes.data, ctypes.byref(sc), ctypes.byref(of))
        return rq, lut, sc.value, of.value

    def qg_scan(self, lut, scale, offset, node):
        qg = self._qg()
        n = int(self.qgf.offsets[node + 1] - self.qgf.offsets[node])
        ds = np.zeros(max(n, 1), np.float32)
        lut = np.ascontiguousarray(lut, np.uint8)
        self.lib.oracle_qg_scan(ctypes.byref(qg), lut.ctypes.data, scale, offset, node, ds.ctypes.data)
        return ds[:n]

    def linear_search(self, queries, k=10, threads=1):
        rows = self.prepare(queries)
        nq = rows.shape[0]
        ids = np.zeros((nq, max(k, 1)), np.uint32)
        ds = np.zeros((nq, max(k, 1)), np.float32)
        n = np.zeros(nq, np.uint32)
        self.lib.oracle_linear_search(ctypes.byref(self.s), rows.ctypes.data, nq, k, ids.ctypes.data,
                                      ds.ctypes.data, n.ctypes.data, threads)
        return ids, ds, n


def rand_sequence(seed: int, n: int) -> np.ndarray:
    lib = ctypes.CDLL(build())
    lib.oracle_rand_sequence.argtypes = [ctypes.c_uint32, ctypes.c_size_t, ctypes.c_void_p]
    out = np.zeros(n, np.int32)
    lib.oracle_rand_sequence(seed, n, out.ctypes.data)
    return out


def write_objects(path: str, rows: np.ndarray) -> None:
    """Writes an NGT object file (dummy slot 0, then one '+' record per row)."""
    rows = np.ascontiguousarray(rows)
    n = rows.shape[0]
    raw = rows.view(np.uint8).reshape(n, -1)
    rec = np.empty((n, 1 + raw.shape[1]), np.uint8)
    rec[:, 0] = ord("+")
    rec[:, 1:] = raw
    with open(path, "wb") as f:
        f.write(np.uint64(n + 1).tobytes())
        f.write(b"-")
        f.write(rec.tobytes())


def read_graph_file(path: str) -> dict:
    """Every node of an NGT graph file (Repository<GraphNode>, lib/NGT/Graph.h:153-160):
    slot count n, presence, CSR offsets (uint64, n+1), edge ids and distances, and the
    trailing prevsize vector's raw bytes (GraphRepository::serialize)."""
    raw = open(path, "rb").read()
    n = int(np.frombuffer(raw, np.uint64, 1, 0)[0])
    pos = 8
    present = np.zeros(n, np.uint8)
    off = np.zeros(n + 1, np.uint64)
    ids, ds = [], []
    total = 0
    for i in range(n):
        t = raw[pos:pos + 1]
        pos += 1
        if t == b"+":
            cnt = int(np.frombuffer(raw, np.uint32, 1, pos)[0])
            pos += 4
            e = np.frombuffer(raw, np.uint32, 2 * cnt, pos).reshape(cnt, 2)
            ids.append(e[:, 0].copy())
            ds.append(e[:, 1].copy().view(np.float32))
            pos += 8 * cnt
            present[i] = 1
            total += cnt
        elif t != b"-":
            raise ValueError("corrupted graph file " + path)
        off[i + 1] = total
    return dict(n=n, present=present, off=off,
                ids=np.concatenate(ids) if ids else np.zeros(0, np.uint32),
                dists=np.concatenate(ds) if ds else np.zeros(0, np.float32), trailer=raw[pos:])


def onng(graph: dict, outgoing: int, incoming: int, min_edges: int = 0, max_edges: int = 2 ** 63 - 1) -> dict:
    """The ONNG of an ANNG graph (read_graph_file's form) as `ngt reconstruct-graph -m S
    -o outgoing -i incoming -E min_edges` builds it (GraphReconstructor::reconstructGraph
    and adjustPathsEffectively): CSR offsets, ids and distances of every node."""
    lib = ctypes.CDLL(build())
    lib.oracle_onng.argtypes = [ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64]
    lib.oracle_onng.restype = ctypes.c_int64
    n = graph["n"]
    cap = len(graph["ids"]) + n * max(incoming, 0) + 1
    off = np.zeros(n + 1, np.uint64)
    ids = np.zeros(cap, np.uint32)
    ds = np.zeros(cap, np.float32)
    present = np.ascontiguousarray(graph["present"], np.uint8)
    goff = np.ascontiguousarray(graph["off"], np.uint64)
    gids = np.ascontiguousarray(graph["ids"], np.uint32)
    gds = np.ascontiguousarray(graph["dists"], np.float32)
    total = lib.oracle_onng(n, present.ctypes.data, goff.ctypes.data, gids.ctypes.data, gds.ctypes.data, outgoing,
                            incoming, max_edges, min_edges, off.ctypes.data, ids.ctypes.data, ds.ctypes.data, cap)
    if total < 0:
        raise RuntimeError("oracle_onng: output buffer too small")
    return dict(n=n, off=off, ids=ids[:total], dists=ds[:total])
