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
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

OBJTYPES = {"Float-4": 0, "Integer-1": 1, "Float-2": 2}
ELEM = {0: np.float32, 1: np.uint8, 2: np.float16}
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


class Oracle:
    """ctypes binding of ngt_oracle.c over one IndexFiles."""

    def __init__(self, files: IndexFiles):
        self.f = files
        self.lib = ctypes.CDLL(build())
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
        L.oracle_distance.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
        L.oracle_distance.restype = ctypes.c_float
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
