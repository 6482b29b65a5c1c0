"""Python mirror of NGT's ctypes wrapper (python/ngt/base.py in the reference)
over libngtgpu.so.

``Index(path, read_only=False)`` opens an existing NGT index directory,
``search(query, k=20, epsilon=0.1)`` returns a list of ``ObjectDistance``
(1-based ids, ascending distance) exactly as the reference's
``ngt.base.Index.search`` does (python/ngt/base.py:281-363).  Errors raised by
the library surface as ``NativeError`` with the library's message.

Extensions (not in the reference wrapper): ``batch_search`` runs many queries
in one native call and returns numpy arrays; ``linear_search`` is the
exhaustive search of the C API.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_bool, c_char_p, c_float, c_int32, c_size_t, c_uint32, c_uint64, c_void_p

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libngtgpu.so")

KERNEL_EXACT = 0
KERNEL_BATCHED = 1
KERNEL_BATCHED_FP32 = 2
KERNEL_WIDE = 3
# tensor-core exhaustive search: score precision and flags (include/ngtgpu.h)
TC_BF16 = 0
TC_FP8 = 1
TC_FP64_TIES = 1
TC_PAIR = 2                # flag: two-CTA clusters share each query tile (TMA multicast)
# QBG search flags (include/ngtq_capi.h)
QBG_TWO_STEP = 1
QBG_REFINE = 2


class NativeError(Exception):
    pass


class ObjectDistance(ctypes.Structure):
    """NGTObjectDistance (lib/NGT/Capi.h:36-39)."""
    _fields_ = [("id", c_uint32), ("distance", c_float)]

    def __repr__(self):
        return "ObjectDistance({},{})".format(self.id, self.distance)


class QueryParameters(ctypes.Structure):
    """NGTQueryParameters (lib/NGT/Capi.h:50-55)."""
    _fields_ = [("size", c_size_t), ("epsilon", c_float), ("radius", c_float), ("edge_size", c_size_t)]


class SearchParameters(ctypes.Structure):
    """NGTGPUSearchParameters (include/ngtgpu.h): NGTQueryParameters with the expected
    accuracy and the refinement expansion of the reference's C++ search container."""
    _fields_ = [("size", c_size_t), ("epsilon", c_float), ("accuracy", c_float), ("radius", c_float),
                ("edge_size", c_size_t), ("refinement_expansion", c_float)]


class QGQueryParameters(ctypes.Structure):
    """NGTQGQueryParameters (lib/NGT/NGTQ/Capi.h:41-46)."""
    _fields_ = [("size", c_size_t), ("epsilon", c_float), ("result_expansion", c_float), ("radius", c_float)]


class QGQueryFloat(ctypes.Structure):
    """NGTQGQueryFloat (lib/NGT/NGTQ/Capi.h:48-51)."""
    _fields_ = [("query", POINTER(c_float)), ("params", QGQueryParameters)]


class QBGQueryParameters(ctypes.Structure):
    """QBGQueryParameters (lib/NGT/NGTQ/Capi.h:129-137)."""
    _fields_ = [("number_of_results", c_size_t), ("epsilon", c_float), ("blob_epsilon", c_float),
                ("result_expansion", c_float), ("number_of_explored_blobs", c_size_t),
                ("number_of_edges", c_size_t), ("radius", c_float)]


class QBGQueryFloat(ctypes.Structure):
    """QBGQueryFloat (lib/NGT/NGTQ/Capi.h:150-153)."""
    _fields_ = [("query", POINTER(c_float)), ("params", QBGQueryParameters)]


class BatchedTuning(ctypes.Structure):
    """NGTGPUBatchedTuning (include/ngtgpu.h)."""
    _fields_ = [("list_capacity", c_uint32), ("parents", c_uint32), ("rerank_factor", c_float),
                ("rows_in_flight", c_uint32), ("ctas_per_sm", c_uint32), ("neighbour_capacity", c_uint32),
                ("cta_threads", c_uint32), ("stage_kilobytes", c_uint32), ("l2_policy", c_uint32),
                ("search_rows", c_uint32)]


class QueryStats(ctypes.Structure):
    _fields_ = [("distance_computations", c_uint32), ("expansions", c_uint32), ("visited", c_uint32),
                ("edges_read", c_uint32), ("status", c_uint32)]


QUERY_STATS_DTYPE = np.dtype([("distance_computations", np.uint32), ("expansions", np.uint32),
                              ("visited", np.uint32), ("edges_read", np.uint32), ("status", np.uint32)])
RESULT_DTYPE = np.dtype([("id", np.uint32), ("distance", np.float32)])

_lib = None


def load_library() -> ctypes.CDLL:
    """Loads libngtgpu.so; raises if it has not been built (there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libngtgpu.so is missing: build it with `python -c 'import __graft_entry__ as g; "
                          "g.build()'` (needs nvcc)")
    L = ctypes.CDLL(LIB_PATH)
    sig = {
        "ngt_open_index": ([c_char_p, c_void_p], c_void_p),
        "ngt_open_index_as_read_only": ([c_char_p, c_void_p], c_void_p),
        "ngt_close_index": ([c_void_p], None),
        "ngt_get_number_of_objects": ([c_void_p, c_void_p], c_uint32),
        "ngt_create_empty_results": ([c_void_p], c_void_p),
        "ngt_search_index": ([c_void_p, POINTER(ctypes.c_double), c_int32, c_size_t, c_float, c_float, c_void_p,
                              c_void_p], c_bool),
        "ngt_search_index_as_float": ([c_void_p, POINTER(c_float), c_int32, c_size_t, c_float, c_float, c_void_p,
                                       c_void_p], c_bool),
        "ngt_search_index_as_uint8": ([c_void_p, POINTER(ctypes.c_uint8), c_int32, c_size_t, c_float, c_float,
                                       c_void_p, c_void_p], c_bool),
        "ngt_linear_search_index_as_float": ([c_void_p, POINTER(c_float), c_int32, c_size_t, c_void_p, c_void_p],
                                             c_bool),
        "ngt_get_result_size": ([c_void_p, c_void_p], c_uint32),
        "ngt_get_result": ([c_void_p, c_uint32, c_void_p], ObjectDistance),
        "ngt_destroy_results": ([c_void_p], None),
        "ngt_create_error_object": ([], c_void_p),
        "ngt_get_error_string": ([c_void_p], c_char_p),
        "ngt_clear_error_string": ([c_void_p], None),
        "ngt_destroy_error_object": ([c_void_p], None),
        "ngt_initialize_query_parameters": ([POINTER(QueryParameters)], None),
        "ngtgpu_get_dimension": ([c_void_p, c_void_p], c_int32),
        "ngtgpu_search_batch_float": ([c_void_p, c_void_p, c_size_t, c_int32, POINTER(QueryParameters), c_size_t,
                                       c_void_p, c_size_t, c_void_p, c_void_p, c_uint32, c_void_p], c_bool),
        "ngtgpu_query_row_bytes": ([c_void_p, c_void_p], c_size_t),
        "ngtgpu_search_batch_ex_float": ([c_void_p, c_void_p, c_size_t, c_int32, POINTER(SearchParameters), c_size_t,
                                          c_void_p, c_size_t, c_void_p, c_void_p, c_uint32, c_void_p], c_bool),
        "ngtgpu_convert_queries_float": ([c_void_p, c_void_p, c_size_t, c_int32, c_void_p, c_void_p], c_bool),
        "ngtgpu_search_batch_device": ([c_void_p, c_void_p, c_size_t, POINTER(QueryParameters), c_size_t, c_void_p,
                                        c_size_t, c_void_p, c_void_p, c_void_p, c_uint32, c_void_p], c_bool),
        "ngtgpu_linear_search_tc_device": ([c_void_p, c_void_p, c_size_t, c_size_t, c_size_t, c_void_p, c_size_t,
                                            c_void_p, c_void_p, c_void_p, c_void_p], c_bool),
        "ngtgpu_linear_search_tc_float": ([c_void_p, c_void_p, c_size_t, c_int32, c_size_t, c_size_t, c_void_p,
                                           c_size_t, c_void_p, c_void_p, c_void_p], c_bool),
        "ngtgpu_linear_search_tc_ex": ([c_void_p, c_void_p, c_size_t, c_size_t, c_size_t, c_uint32, c_uint32,
                                        c_void_p, c_size_t, c_void_p, c_void_p, c_void_p, c_void_p], c_bool),
        "ngtgpu_linear_search_tc_float_ex": ([c_void_p, c_void_p, c_size_t, c_int32, c_size_t, c_size_t, c_uint32,
                                              c_uint32, c_void_p, c_size_t, c_void_p, c_void_p, c_void_p], c_bool),
        "ngtgpu_tc_scores_device": ([c_void_p, c_void_p, c_size_t, c_void_p, c_size_t, c_void_p, c_void_p],
                                    c_bool),
        "ngtgpu_set_tc_first_rows": ([c_void_p, c_size_t, c_void_p], c_bool),
        "ngtgpu_set_tc_graphs": ([c_void_p, c_int32, c_void_p], c_bool),
        "ngtgpu_tc_phase_times": ([c_void_p, c_void_p, c_void_p], c_bool),
        "ngtgpu_kernel_launches": ([c_void_p, c_void_p], c_uint64),
        "ngtgpu_coalescing_stats": ([c_void_p, c_void_p, c_void_p, c_void_p], c_bool),
        "ngtgpu_set_tc_row_range": ([c_void_p, c_size_t, c_size_t, c_void_p], c_bool),
        "ngtgpu_autotune": ([c_void_p, c_void_p, c_size_t, c_int32, c_size_t, c_float, c_float,
                             POINTER(BatchedTuning), c_void_p, c_void_p, c_void_p, c_void_p], c_bool),
        "ngtgpu_get_wide_search_rows": ([c_void_p, c_void_p], c_uint32),
        "ngtgpu_set_batched_tuning": ([c_void_p, c_uint32, c_uint32, c_float, c_void_p], c_bool),
        "ngtgpu_set_batched_rows_in_flight": ([c_void_p, c_uint32, c_void_p], c_bool),
        "ngtgpu_set_batched_tuning_ex": ([c_void_p, POINTER(BatchedTuning), c_void_p], c_bool),
        "ngtgpu_server_create": ([c_void_p, c_uint32, c_uint32, c_uint32, c_void_p], c_void_p),
        "ngtgpu_server_create_ex": ([c_void_p, c_uint32, c_uint32, c_uint32, c_uint32, c_void_p], c_void_p),
        "ngtgpu_server_submit": ([c_void_p, c_void_p, c_size_t, c_int32, POINTER(QueryParameters), c_size_t,
                                  c_void_p], ctypes.c_int64),
        "ngtgpu_server_wait": ([c_void_p, ctypes.c_int64, c_void_p, c_size_t, c_void_p, POINTER(ctypes.c_double),
                                c_void_p], c_bool),
        "ngtgpu_server_destroy": ([c_void_p], None),
        "ngtgpu_build_onng": ([c_char_p, c_char_p, c_int32, c_int32, ctypes.c_int64, c_void_p], c_bool),
        "ngtgpu_set_coalescing_lanes": ([c_void_p, c_uint32, c_void_p], c_bool),
        "ngtgpu_server_submit_deadline": ([c_void_p, c_void_p, c_size_t, c_int32, POINTER(QueryParameters),
                                           c_size_t, ctypes.c_double, c_void_p], ctypes.c_int64),
        "ngtgpu_server_set_deadline": ([c_void_p, ctypes.c_double, c_void_p], c_bool),
        "ngtgpu_server_cancel": ([c_void_p, ctypes.c_int64, c_void_p], c_bool),
        "ngtgpu_qg_server_create": ([c_void_p, c_uint32, c_uint32, c_uint32, c_void_p], c_void_p),
        "ngtgpu_qg_server_create_ex": ([c_void_p, c_uint32, c_uint32, c_uint32, c_uint32, c_void_p], c_void_p),
        "ngtgpu_qg_server_submit": ([c_void_p, c_void_p, c_size_t, c_int32, POINTER(QGQueryParameters), c_size_t,
                                     c_void_p], ctypes.c_int64),
        "ngtgpu_qbg_server_create": ([c_void_p, c_uint32, c_uint32, c_uint32, c_uint32, c_void_p], c_void_p),
        "ngtgpu_qbg_server_submit": ([c_void_p, c_void_p, c_size_t, c_int32, POINTER(QBGQueryParameters), c_size_t,
                                      c_void_p], ctypes.c_int64),
        "ngtqg_open_index": ([c_char_p, c_void_p], c_void_p),
        "ngtqg_close_index": ([c_void_p], None),
        "ngtqg_initialize_query_parameters": ([POINTER(QGQueryParameters)], None),
        "ngtqg_search_index_float": ([c_void_p, QGQueryFloat, c_void_p, c_void_p], c_bool),
        "ngtqg_gpu_search_batch_float": ([c_void_p, c_void_p, c_size_t, c_int32, POINTER(QGQueryParameters),
                                          c_size_t, c_void_p, c_size_t, c_void_p, c_void_p, c_void_p], c_bool),
        "ngtqg_gpu_search_batch_ex_float": ([c_void_p, c_void_p, c_size_t, c_int32, POINTER(QGQueryParameters),
                                             c_size_t, c_void_p, c_size_t, c_void_p, c_void_p, c_uint32, c_void_p],
                                            c_bool),
        "ngtqg_gpu_search_batch_ex_device": ([c_void_p, c_void_p, c_size_t, POINTER(QGQueryParameters), c_size_t,
                                              c_void_p, c_size_t, c_void_p, c_void_p, c_void_p, c_uint32, c_void_p],
                                             c_bool),
        "ngtqg_gpu_search_batch_device": ([c_void_p, c_void_p, c_size_t, POINTER(QGQueryParameters), c_size_t,
                                           c_void_p, c_size_t, c_void_p, c_void_p, c_void_p, c_void_p], c_bool),
        "qbg_open_index": ([c_char_p, c_bool, c_void_p], c_void_p),
        "qbg_close_index": ([c_void_p], None),
        "qbg_get_dimension": ([c_void_p, c_void_p], c_size_t),
        "qbg_initialize_query_parameters": ([POINTER(QBGQueryParameters)], None),
        "qbg_search_index_float": ([c_void_p, QBGQueryFloat, c_void_p, c_void_p], c_bool),
        "qbg_gpu_search_batch_float": ([c_void_p, c_void_p, c_size_t, c_int32, POINTER(QBGQueryParameters),
                                        c_size_t, c_void_p, c_size_t, c_void_p, c_void_p, c_void_p], c_bool),
        "qbg_gpu_search_batch_ex": ([c_void_p, c_void_p, c_size_t, c_int32, POINTER(QBGQueryParameters),
                                     c_size_t, c_uint32, c_void_p, c_size_t, c_void_p, c_void_p, c_void_p], c_bool),
        "qbg_gpu_search_batch_device": ([c_void_p, c_void_p, c_size_t, POINTER(QBGQueryParameters), c_size_t,
                                         c_uint32, c_void_p, c_size_t, c_void_p, c_void_p, c_void_p, c_void_p],
                                        c_bool),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def build_onng(anng_index: str, onng_index: str, outgoing: int = -1, incoming: int = -1, min_edges: int = 0):
    """`ngt reconstruct-graph -m S -o outgoing -i incoming -E min_edges` on the GPU:
    copies anng_index to onng_index (which must not exist) and rebuilds its graph as
    the reference's ONNG reconstruction and path adjustment do (ngtgpu_build_onng)."""
    L = load_library()
    err = L.ngt_create_error_object()
    try:
        if not L.ngtgpu_build_onng(anng_index.encode(), onng_index.encode(), outgoing, incoming, min_edges, err):
            raise NativeError(L.ngt_get_error_string(err).decode())
    finally:
        L.ngt_destroy_error_object(err)


def _edge_field(edge_size):
    """NGTQueryParameters.edge_size: INT_MIN (stored in a size_t) = index default."""
    if edge_size is None or edge_size == -1:
        return ctypes.c_size_t(-2147483648).value
    return ctypes.c_size_t(int(edge_size)).value


class Index:
    """An NGT index opened on the GPU (mirror of ngt.base.Index)."""

    def __init__(self, path: str, read_only: bool = False):
        self._lib = load_library()
        self._err = self._lib.ngt_create_error_object()
        opener = self._lib.ngt_open_index_as_read_only if read_only else self._lib.ngt_open_index
        self._index = opener(path.encode(), self._err)
        self._check(self._index is not None)
        self.dimension = self._lib.ngtgpu_get_dimension(self._index, self._err)
        self._results = self._lib.ngt_create_empty_results(self._err)

    def _check(self, ok):
        if not ok:
            msg = self._lib.ngt_get_error_string(self._err).decode()
            self._lib.ngt_clear_error_string(self._err)
            raise NativeError(msg)

    def close(self):
        if getattr(self, "_index", None):
            self._lib.ngt_close_index(self._index)
            self._index = None
        if getattr(self, "_results", None):
            self._lib.ngt_destroy_results(self._results)
            self._results = None
        if getattr(self, "_err", None):
            self._lib.ngt_destroy_error_object(self._err)
            self._err = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _collect(self):
        n = self._lib.ngt_get_result_size(self._results, self._err)
        return [self._lib.ngt_get_result(self._results, i, self._err) for i in range(n)]

    def search(self, query, k: int = 20, epsilon: float = 0.1, radius: float = -1.0):
        """Graph search of one query: list of ObjectDistance (id, distance).  Safe to call
        from several threads at once: each call has its own result and error objects
        (the library coalesces concurrent calls into one launch)."""
        q = np.ascontiguousarray(query, dtype=np.float32)
        L = self._lib
        err = L.ngt_create_error_object()
        res = L.ngt_create_empty_results(err)
        try:
            ok = L.ngt_search_index_as_float(self._index, q.ctypes.data_as(POINTER(c_float)), q.shape[0], k,
                                             epsilon, radius, res, err)
            if not ok:
                raise NativeError(L.ngt_get_error_string(err).decode())
            n = L.ngt_get_result_size(res, err)
            return [L.ngt_get_result(res, i, err) for i in range(n)]
        finally:
            L.ngt_destroy_results(res)
            L.ngt_destroy_error_object(err)

    def linear_search(self, query, k: int = 20):
        q = np.ascontiguousarray(query, dtype=np.float32)
        ok = self._lib.ngt_linear_search_index_as_float(self._index, q.ctypes.data_as(POINTER(c_float)),
                                                        q.shape[0], k, self._results, self._err)
        self._check(ok)
        return self._collect()

    def number_of_objects(self) -> int:
        return self._lib.ngt_get_number_of_objects(self._index, self._err)

    @staticmethod
    def make_params(k, epsilon, radius=-1.0, edge_size=None):
        """Per-query NGTQueryParameters array from scalars or sequences."""
        ks, es, rs, eds = (np.atleast_1d(np.asarray(x)) for x in (k, epsilon, radius,
                                                                  -1 if edge_size is None else edge_size))
        n = max(len(ks), len(es), len(rs), len(eds))
        arr = (QueryParameters * n)()
        for i in range(n):
            arr[i].size = int(ks[i % len(ks)])
            arr[i].epsilon = float(es[i % len(es)])
            arr[i].radius = float(rs[i % len(rs)])
            arr[i].edge_size = _edge_field(int(eds[i % len(eds)]))
        return arr, n

    def batch_search(self, queries, k=10, epsilon=0.1, radius=-1.0, edge_size=None, kernel: int = KERNEL_EXACT,
                     with_stats: bool = False):
        """Searches every row of `queries` in one native call.

        k / epsilon / radius / edge_size may be scalars or per-query sequences.
        Returns (ids[nq, kmax], distances[nq, kmax], counts[nq]) and, with
        with_stats, the per-query counters.
        """
        q = np.ascontiguousarray(queries, dtype=np.float32)
        nq = q.shape[0]
        params, n = self.make_params(k, epsilon, radius, edge_size)
        # room for round((1+epsilon)*k): the updatable search on an index with
        # EpsilonType ResultSize returns that many results
        kmax = int(np.ceil(max(np.atleast_1d(k)) * (1.0 + max(0.0, float(np.max(epsilon)))))) + 1
        res = np.zeros((nq, kmax), RESULT_DTYPE)
        counts = np.zeros(nq, np.uint32)
        stats = np.zeros(nq, QUERY_STATS_DTYPE)
        ok = self._lib.ngtgpu_search_batch_float(self._index, q.ctypes.data, nq, q.shape[1], params, n,
                                                 res.ctypes.data, kmax, counts.ctypes.data, stats.ctypes.data,
                                                 kernel, self._err)
        self._check(ok)
        m = int(counts.max()) if nq else 0
        out = (res["id"][:, :m].copy(), res["distance"][:, :m].copy(), counts)
        return out + (stats,) if with_stats else out

    def batch_search_accuracy(self, queries, k=10, accuracy=0.9, epsilon=0.1, radius=-1.0, edge_size=None,
                              kernel: int = KERNEL_EXACT):
        """batch_search with the expected accuracy of the reference's C++ search container:
        epsilon comes from the index's AccuracyTable (ngtgpu_search_batch_ex_float)."""
        q = np.ascontiguousarray(queries, dtype=np.float32)
        nq = q.shape[0]
        p = SearchParameters(int(k), float(epsilon), float(accuracy), float(radius),
                             _edge_field(-1 if edge_size is None else edge_size), 0.0)
        return self._search_ex(q, p, int(np.ceil(k * 1.4)) + 1, kernel)

    def batch_search_refined(self, queries, k=10, expansion=2.0, epsilon=0.1, edge_size=None,
                             kernel: int = KERNEL_EXACT):
        """batch_search with the refinement expansion of the reference's C++ search
        container: k x expansion results re-ranked by exact distances over the index's
        refinement objects (robj) to the k best (ngtgpu_search_batch_ex_float)."""
        q = np.ascontiguousarray(queries, dtype=np.float32)
        p = SearchParameters(int(k), float(epsilon), -1.0, -1.0,
                             _edge_field(-1 if edge_size is None else edge_size), float(expansion))
        return self._search_ex(q, p, int(k), kernel)

    def _search_ex(self, q, p, kmax, kernel):
        nq = q.shape[0]
        res = np.zeros((nq, kmax), RESULT_DTYPE)
        counts = np.zeros(nq, np.uint32)
        L = self._lib
        err = L.ngt_create_error_object()
        try:
            ok = L.ngtgpu_search_batch_ex_float(self._index, q.ctypes.data, nq, q.shape[1], ctypes.byref(p), 1,
                                                res.ctypes.data, kmax, counts.ctypes.data, None, kernel, err)
            if not ok:
                raise NativeError(L.ngt_get_error_string(err).decode())
        finally:
            L.ngt_destroy_error_object(err)
        m = int(counts.max()) if nq else 0
        return res["id"][:, :m].copy(), res["distance"][:, :m].copy(), counts

    def set_batched_tuning(self, list_capacity: int = 0, parents: int = 0, rerank_factor: float = 0.0,
                           rows_in_flight: int = 0, ctas_per_sm: int = 0, neighbour_capacity: int = 0,
                           cta_threads: int = 0, stage_kilobytes: int = 0, l2_policy: int = 0,
                           search_rows: int = 0):
        t = BatchedTuning(list_capacity, parents, rerank_factor, rows_in_flight, ctas_per_sm, neighbour_capacity,
                          cta_threads, stage_kilobytes, l2_policy, search_rows)
        self._check(self._lib.ngtgpu_set_batched_tuning_ex(self._index, ctypes.byref(t), self._err))

    def linear_search_tc(self, queries, k: int = 10, candidates: int = 0, first_rows: int = 0,
                         precision: str = "bf16", fp64_ties: bool = False, pair: bool = False):
        """Exhaustive k-NN of every row of `queries` with the tensor-core
        pre-selection (bf16 or per-row scaled fp8 scores, `candidates` re-ranked
        exactly; fp64_ties: the ties at the cut ordered by FP64 distance).

        Returns (ids[nq, k], distances[nq, k], counts[nq], status[nq]); status
        bit 1 marks a query whose candidate list overflowed, bit 4 a tie window
        too wide for the FP64 check.
        """
        q = np.ascontiguousarray(queries, dtype=np.float32)
        nq = q.shape[0]
        self._check(self._lib.ngtgpu_set_tc_first_rows(self._index, first_rows, self._err))
        res = np.zeros((nq, k), RESULT_DTYPE)
        counts = np.zeros(nq, np.uint32)
        status = np.zeros(nq, np.uint32)
        prec = {"bf16": TC_BF16, "fp8": TC_FP8}[precision]
        ok = self._lib.ngtgpu_linear_search_tc_float_ex(self._index, q.ctypes.data, nq, q.shape[1], k, candidates,
                                                        prec, (TC_FP64_TIES if fp64_ties else 0) |
                                                        (TC_PAIR if pair else 0), res.ctypes.data, k,
                                                        counts.ctypes.data, status.ctypes.data, self._err)
        self._check(ok)
        return res["id"].copy(), res["distance"].copy(), counts, status

    def set_tc_graphs(self, enable: bool = True) -> None:
        """Replay captured CUDA graphs of the tensor-core search's launch sequence
        (one per shape, buffers and options) instead of launching it each call."""
        self._check(self._lib.ngtgpu_set_tc_graphs(self._index, 1 if enable else 0, self._err))

    def tc_phase_times(self):
        """CUDA-event milliseconds of the last tensor-core search batch: (dense
        part + selection, filtered part, final re-rank)."""
        ms = np.zeros(3, np.float32)
        self._check(self._lib.ngtgpu_tc_phase_times(self._index, ms.ctypes.data, self._err))
        return tuple(float(v) for v in ms)

    def tc_scores(self, queries) -> np.ndarray:
        """Approximate scores [nq, number of object slots] of the tensor-core
        pre-selection (larger = closer; -inf for id 0 and removed objects)."""
        import torch
        rows = torch.from_numpy(self.convert_queries(queries)).cuda()
        nq = rows.shape[0]
        nslots = self.number_of_objects() + 1
        out = torch.empty((nq, nslots), dtype=torch.float32, device="cuda")
        ok = self._lib.ngtgpu_tc_scores_device(self._index, rows.data_ptr(), nq, out.data_ptr(), nslots, None,
                                               self._err)
        self._check(ok)
        return out.cpu().numpy()

    def kernel_launches(self) -> int:
        return int(self._lib.ngtgpu_kernel_launches(self._index, self._err))

    def autotune(self, queries, k: int = 10, epsilon: float = 0.1, recall_floor: float = -1.0):
        """ngtgpu_autotune: the fastest batched configuration for (k, epsilon) on these
        sample queries whose recall reaches the floor (default: the exact-order
        kernel's; epsilon < 0: each configuration at the smallest epsilon of a sweep
        reaching the floor).  It becomes the index's tuning; returns (kernel, tuning
        fields, qps on the sample, epsilon)."""
        q = np.ascontiguousarray(queries, dtype=np.float32)
        t = BatchedTuning()
        kern, qps, eps = ctypes.c_uint32(0), ctypes.c_float(0.0), ctypes.c_float(0.0)
        self._check(self._lib.ngtgpu_autotune(self._index, q.ctypes.data, q.shape[0], q.shape[1], k, epsilon,
                                              recall_floor, ctypes.byref(t), ctypes.byref(kern), ctypes.byref(qps),
                                              ctypes.byref(eps), self._err))
        fields = {name: getattr(t, name) for name, _ in BatchedTuning._fields_}
        return int(kern.value), fields, float(qps.value), float(eps.value)

    def coalescing_stats(self):
        """(queries, launches) of the coalesced single-query calls so far."""
        q, n = ctypes.c_uint64(0), ctypes.c_uint64(0)
        self._check(self._lib.ngtgpu_coalescing_stats(self._index, ctypes.byref(q), ctypes.byref(n), self._err))
        return int(q.value), int(n.value)

    def wide_search_rows(self) -> str:
        """Search rows of the CTA-per-query kernel: "native", "bf16" or "u8"."""
        v = int(self._lib.ngtgpu_get_wide_search_rows(self._index, self._err))
        if v == 0xFFFFFFFF:
            self._check(False)
        return ("native", "bf16", "u8")[v]

    # device-resident path (used by bench.py for the HBM-resident measurement)
    def query_row_bytes(self) -> int:
        return int(self._lib.ngtgpu_query_row_bytes(self._index, self._err))

    def convert_queries(self, queries) -> np.ndarray:
        q = np.ascontiguousarray(queries, dtype=np.float32)
        rows = np.zeros((q.shape[0], self.query_row_bytes()), np.uint8)
        self._check(self._lib.ngtgpu_convert_queries_float(self._index, q.ctypes.data, q.shape[0], q.shape[1],
                                                           rows.ctypes.data, self._err))
        return rows

    def search_device(self, d_rows: int, nq: int, params, nparams: int, d_results: int, kmax: int, d_counts: int,
                      d_stats: int, stream: int = 0, kernel: int = KERNEL_EXACT):
        ok = self._lib.ngtgpu_search_batch_device(self._index, d_rows, nq, params, nparams, d_results, kmax,
                                                  d_counts, d_stats, stream or None, kernel, self._err)
        self._check(ok)


class QuantizedIndex:
    """A quantized-graph index opened on the GPU: mirror of ngtpy.QuantizedIndex
    (python/src/ngtpy.cpp:573-700) over the ngtqg_* C API.

    ``search(query, size, epsilon, result_expansion)`` returns a list of
    (id, distance) tuples, ids zero-based unless zero_based_numbering=False;
    unset arguments take the defaults (size 20, epsilon 0.02, result
    expansion 3.0, no radius).  The index needs a quantized graph built by the
    reference (`qbg create-qg` + `qbg build-qg`).
    """

    def __init__(self, path: str, max_no_of_edges: int = 128, zero_based_numbering: bool = True,
                 tree_disabled: bool = False, log_disabled: bool = False):
        if tree_disabled:
            raise NativeError("tree_disabled=True is not supported: seeds come from the tree when it exists")
        self._lib = load_library()
        self._err = self._lib.ngt_create_error_object()
        self._index = self._lib.ngtqg_open_index(path.encode(), self._err)
        if not self._index:
            raise NativeError(self._lib.ngt_get_error_string(self._err).decode())
        self._results = self._lib.ngt_create_empty_results(self._err)
        self.dimension = self._lib.ngtgpu_get_dimension(self._index, self._err)
        self.zero = 1 if zero_based_numbering else 0
        self.defaults = dict(size=20, epsilon=0.02, result_expansion=3.0, radius=-1.0)

    def _check(self, ok):
        if not ok:
            msg = self._lib.ngt_get_error_string(self._err).decode()
            self._lib.ngt_clear_error_string(self._err)
            raise NativeError(msg)

    def set(self, num_of_search_objects=0, radius=-1.0, epsilon=-float("inf"), result_expansion=-1.0):
        """QuantizedIndex.set (python/src/ngtpy.cpp:674-693)."""
        if num_of_search_objects > 0:
            self.defaults["size"] = num_of_search_objects
        if epsilon > -1.0:
            self.defaults["epsilon"] = epsilon
        if radius >= 0.0:
            self.defaults["radius"] = radius
        if result_expansion >= 0.0:
            self.defaults["result_expansion"] = result_expansion

    def _params(self, size, epsilon, result_expansion):
        p = QGQueryParameters()
        p.size = int(size) if size and size > 0 else self.defaults["size"]
        p.epsilon = float(epsilon) if epsilon is not None and epsilon > -1.0 else self.defaults["epsilon"]
        p.result_expansion = (float(result_expansion) if result_expansion is not None and result_expansion >= 0.0
                              else self.defaults["result_expansion"])
        p.radius = self.defaults["radius"]
        return p

    def search(self, query, size=0, epsilon=None, result_expansion=None):
        q = np.ascontiguousarray(query, dtype=np.float32)
        qq = QGQueryFloat()
        qq.query = q.ctypes.data_as(POINTER(c_float))
        qq.params = self._params(size, epsilon, result_expansion)
        self._check(self._lib.ngtqg_search_index_float(self._index, qq, self._results, self._err))
        n = self._lib.ngt_get_result_size(self._results, self._err)
        out = []
        for i in range(n):
            r = self._lib.ngt_get_result(self._results, i, self._err)
            out.append((r.id - self.zero, r.distance))
        return out

    def batch_search(self, queries, size=0, epsilon=None, result_expansion=None, with_stats: bool = False,
                     kernel: int = KERNEL_EXACT):
        """Every row of `queries` in one launch: (ids[nq, m], distances[nq, m], counts[nq]),
        ids as stored (1-based).  kernel: KERNEL_EXACT (the reference's order) or
        KERNEL_WIDE (relaxed order, several parents per step)."""
        q = np.ascontiguousarray(queries, dtype=np.float32)
        nq = q.shape[0]
        p = self._params(size, epsilon, result_expansion)
        kmax = max(int(p.size), 1)
        res = np.zeros((nq, kmax), RESULT_DTYPE)
        counts = np.zeros(nq, np.uint32)
        stats = np.zeros(nq, QUERY_STATS_DTYPE)
        ok = self._lib.ngtqg_gpu_search_batch_ex_float(self._index, q.ctypes.data, nq, q.shape[1], ctypes.byref(p),
                                                       1, res.ctypes.data, kmax, counts.ctypes.data,
                                                       stats.ctypes.data, kernel, self._err)
        self._check(ok)
        m = int(counts.max()) if nq else 0
        out = (res["id"][:, :m].copy(), res["distance"][:, :m].copy(), counts)
        return out + (stats,) if with_stats else out

    def search_device(self, d_rows: int, nq: int, params, d_results: int, kmax: int, d_counts: int, d_stats: int,
                      stream: int = 0, kernel: int = KERNEL_EXACT):
        ok = self._lib.ngtqg_gpu_search_batch_ex_device(self._index, d_rows, nq, ctypes.byref(params), 1, d_results,
                                                        kmax, d_counts, d_stats, stream or None, kernel, self._err)
        self._check(ok)

    def set_batched_tuning(self, list_capacity: int = 0, parents: int = 0, blocks_in_flight: int = 0):
        """Parents per step, list capacity and code blocks each warp loads at a time (2 or
        4) of the relaxed-order kernel (0: automatic)."""
        t = BatchedTuning(list_capacity, parents, 0.0, blocks_in_flight, 0, 0, 0, 0, 0, 0)
        self._check(self._lib.ngtgpu_set_batched_tuning_ex(self._index, ctypes.byref(t), self._err))

    def convert_queries(self, queries) -> np.ndarray:
        q = np.ascontiguousarray(queries, dtype=np.float32)
        rb = int(self._lib.ngtgpu_query_row_bytes(self._index, self._err))
        rows = np.zeros((q.shape[0], rb), np.uint8)
        self._check(self._lib.ngtgpu_convert_queries_float(self._index, q.ctypes.data, q.shape[0], q.shape[1],
                                                           rows.ctypes.data, self._err))
        return rows

    def kernel_launches(self) -> int:
        return int(self._lib.ngtgpu_kernel_launches(self._index, self._err))

    def close(self):
        if getattr(self, "_index", None):
            self._lib.ngtqg_close_index(self._index)
            self._index = None
        if getattr(self, "_results", None):
            self._lib.ngt_destroy_results(self._results)
            self._results = None
        if getattr(self, "_err", None):
            self._lib.ngt_destroy_error_object(self._err)
            self._err = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class QBGIndex:
    """A quantized-blob-graph index opened on the GPU through the reference's QBG
    C API (qbg_open_index / qbg_search_index_float, lib/NGT/NGTQ/Capi.h).

    ``search(query, k, ...)`` returns a list of ObjectDistance (1-based ids,
    ascending), k x result_expansion of them with quantized distances when the
    expansion is >= 1, exactly as qbg_search_index_float does.
    """

    def __init__(self, path: str):
        self._lib = load_library()
        self._err = self._lib.ngt_create_error_object()
        self._index = self._lib.qbg_open_index(path.encode(), True, self._err)
        if not self._index:
            raise NativeError(self._lib.ngt_get_error_string(self._err).decode())
        self._results = self._lib.ngt_create_empty_results(self._err)
        self.dimension = int(self._lib.qbg_get_dimension(self._index, self._err))

    def _check(self, ok):
        if not ok:
            msg = self._lib.ngt_get_error_string(self._err).decode()
            self._lib.ngt_clear_error_string(self._err)
            raise NativeError(msg)

    @staticmethod
    def params(k=20, epsilon=0.1, blob_epsilon=0.0, result_expansion=3.0, explored_blobs=256, edges=0):
        p = QBGQueryParameters()
        p.number_of_results, p.epsilon, p.blob_epsilon = int(k), float(epsilon), float(blob_epsilon)
        p.result_expansion, p.number_of_explored_blobs = float(result_expansion), int(explored_blobs)
        p.number_of_edges, p.radius = int(edges), 0.0
        return p

    @staticmethod
    def result_size(p) -> int:
        return int(np.float32(p.number_of_results) * np.float32(p.result_expansion)) \
            if p.result_expansion >= 1.0 else int(p.number_of_results)

    def search(self, query, k=20, epsilon=0.1, blob_epsilon=0.0, result_expansion=3.0, explored_blobs=256, edges=0):
        q = np.ascontiguousarray(query, dtype=np.float32)
        qq = QBGQueryFloat()
        qq.query = q.ctypes.data_as(POINTER(c_float))
        qq.params = self.params(k, epsilon, blob_epsilon, result_expansion, explored_blobs, edges)
        self._check(self._lib.qbg_search_index_float(self._index, qq, self._results, self._err))
        n = self._lib.ngt_get_result_size(self._results, self._err)
        return [self._lib.ngt_get_result(self._results, i, self._err) for i in range(n)]

    def batch_search(self, queries, k=20, epsilon=0.1, blob_epsilon=0.0, result_expansion=3.0, explored_blobs=256,
                     edges=0, with_stats: bool = False, two_step: bool = False, refine: bool = False):
        """Every row in one launch: (ids[nq, m], distances[nq, m], counts[nq]).

        two_step: searchInTwoSteps (explored_blobs probes); refine: result_expansion is
        the refinement expansion (exact re-rank over the object list to k results)."""
        q = np.ascontiguousarray(queries, dtype=np.float32)
        nq = q.shape[0]
        p = self.params(k, epsilon, blob_epsilon, result_expansion, explored_blobs, edges)
        kmax = max(int(k) if refine and result_expansion >= 1.0 else self.result_size(p), 1)
        res = np.zeros((nq, kmax), RESULT_DTYPE)
        counts = np.zeros(nq, np.uint32)
        stats = np.zeros(nq, QUERY_STATS_DTYPE)
        flags = (QBG_TWO_STEP if two_step else 0) | (QBG_REFINE if refine else 0)
        self._check(self._lib.qbg_gpu_search_batch_ex(self._index, q.ctypes.data, nq, q.shape[1],
                                                      ctypes.byref(p), 1, flags, res.ctypes.data, kmax,
                                                      counts.ctypes.data, stats.ctypes.data, self._err))
        m = int(counts.max()) if nq else 0
        out = (res["id"][:, :m].copy(), res["distance"][:, :m].copy(), counts)
        return out + (stats,) if with_stats else out

    def close(self):
        if getattr(self, "_index", None):
            self._lib.qbg_close_index(self._index)
            self._index = None
        if getattr(self, "_results", None):
            self._lib.ngt_destroy_results(self._results)
            self._results = None
        if getattr(self, "_err", None):
            self._lib.ngt_destroy_error_object(self._err)
            self._err = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class QBGServer:
    """The continuous-batching serving loop over an open QBGIndex
    (ngtgpu_qbg_server_*): every request runs the one-step search of the C API, or
    with two_step / refine the reference's searchInTwoSteps / refinement."""

    def __init__(self, index: "QBGIndex", max_batch: int = 1024, inflight: int = 3, max_k: int = 128,
                 two_step: bool = False, refine: bool = False):
        self._ix = index
        self._lib = index._lib
        self._err = self._lib.ngt_create_error_object()
        flags = (QBG_TWO_STEP if two_step else 0) | (QBG_REFINE if refine else 0)
        self._srv = self._lib.ngtgpu_qbg_server_create(index._index, max_batch, inflight, max_k, flags, self._err)
        if not self._srv:
            raise NativeError(self._lib.ngt_get_error_string(self._err).decode())
        self.max_k = max_k
        self._pending = {}

    def submit(self, queries, k=20, epsilon=0.1, blob_epsilon=0.0, result_expansion=3.0, explored_blobs=256,
               edges=0) -> int:
        q = np.ascontiguousarray(queries, dtype=np.float32)
        if q.ndim == 1:
            q = q[None, :]
        p = QBGIndex.params(k, epsilon, blob_epsilon, result_expansion, explored_blobs, edges)
        t = self._lib.ngtgpu_qbg_server_submit(self._srv, q.ctypes.data, q.shape[0], q.shape[1], ctypes.byref(p), 1,
                                               self._err)
        if t < 0:
            raise NativeError(self._lib.ngt_get_error_string(self._err).decode())
        self._pending[t] = q.shape[0]
        return t

    def wait(self, ticket: int, kmax: int | None = None):
        return Server.wait(self, ticket, kmax)

    def cancel(self, ticket: int) -> bool:
        return Server.cancel(self, ticket)

    def set_deadline(self, deadline_ms: float):
        Server.set_deadline(self, deadline_ms)

    def close(self):
        Server.close(self)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class QGServer:
    """The continuous-batching serving loop over an open QuantizedIndex
    (ngtgpu_qg_server_*): every request runs ngtqg_search_index_float's search."""

    def __init__(self, index: "QuantizedIndex", max_batch: int = 1024, inflight: int = 3, max_k: int = 128,
                 kernel: int = KERNEL_EXACT):
        self._ix = index
        self._lib = index._lib
        self._err = self._lib.ngt_create_error_object()
        self._srv = self._lib.ngtgpu_qg_server_create_ex(index._index, max_batch, inflight, max_k, kernel, self._err)
        if not self._srv:
            raise NativeError(self._lib.ngt_get_error_string(self._err).decode())
        self.max_k = max_k
        self._pending = {}

    def submit(self, queries, k=20, epsilon=0.03, result_expansion=3.0, radius=-1.0) -> int:
        q = np.ascontiguousarray(queries, dtype=np.float32)
        if q.ndim == 1:
            q = q[None, :]
        p = QGQueryParameters(int(k), float(epsilon), float(result_expansion), float(radius))
        t = self._lib.ngtgpu_qg_server_submit(self._srv, q.ctypes.data, q.shape[0], q.shape[1], ctypes.byref(p), 1,
                                              self._err)
        if t < 0:
            raise NativeError(self._lib.ngt_get_error_string(self._err).decode())
        self._pending[t] = q.shape[0]
        return t

    def wait(self, ticket: int, kmax: int | None = None):
        return Server.wait(self, ticket, kmax)

    def cancel(self, ticket: int) -> bool:
        return Server.cancel(self, ticket)

    def set_deadline(self, deadline_ms: float):
        Server.set_deadline(self, deadline_ms)

    def close(self):
        Server.close(self)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Server:
    """Continuous-batching serving loop over an open Index (ngtgpu_server_*)."""

    def __init__(self, index: Index, max_batch: int = 4096, inflight: int = 3, max_k: int = 128,
                 kernel: int = KERNEL_BATCHED):
        self._ix = index
        self._lib = index._lib
        self._err = self._lib.ngt_create_error_object()
        self._srv = self._lib.ngtgpu_server_create_ex(index._index, max_batch, inflight, max_k, kernel, self._err)
        if not self._srv:
            raise NativeError(self._lib.ngt_get_error_string(self._err).decode())
        self.max_k = max_k
        self._pending = {}

    def submit(self, queries, k=10, epsilon=0.1, radius=-1.0, edge_size=None, deadline_ms=None) -> int:
        """Queues a request; deadline_ms: it must be launched within that time of now,
        else its wait raises "deadline exceeded before launch"."""
        q = np.ascontiguousarray(queries, dtype=np.float32)
        if q.ndim == 1:
            q = q[None, :]
        params, n = Index.make_params(k, epsilon, radius, edge_size)
        if deadline_ms is None:
            t = self._lib.ngtgpu_server_submit(self._srv, q.ctypes.data, q.shape[0], q.shape[1], params, n,
                                               self._err)
        else:
            t = self._lib.ngtgpu_server_submit_deadline(self._srv, q.ctypes.data, q.shape[0], q.shape[1], params, n,
                                                        float(deadline_ms), self._err)
        if t < 0:
            raise NativeError(self._lib.ngt_get_error_string(self._err).decode())
        self._pending[t] = q.shape[0]
        return t

    def cancel(self, ticket: int) -> bool:
        """Withdraws a request not yet launched (True; its wait then raises "cancelled")."""
        self._lib.ngt_clear_error_string(self._err)
        ok = self._lib.ngtgpu_server_cancel(self._srv, ticket, self._err)
        if not ok:
            msg = self._lib.ngt_get_error_string(self._err).decode()
            self._lib.ngt_clear_error_string(self._err)
            if msg:
                raise NativeError(msg)
        return bool(ok)

    def set_deadline(self, deadline_ms: float):
        """Default admission deadline of later submits (<= 0: none)."""
        self._lib.ngtgpu_server_set_deadline(self._srv, float(deadline_ms), self._err)

    def wait(self, ticket: int, kmax: int | None = None):
        nq = self._pending.pop(ticket)
        if self._err:
            self._lib.ngt_clear_error_string(self._err)
        kmax = kmax or self.max_k
        res = np.zeros((nq, kmax), RESULT_DTYPE)
        counts = np.zeros(nq, np.uint32)
        lat = ctypes.c_double(0.0)
        ok = self._lib.ngtgpu_server_wait(self._srv, ticket, res.ctypes.data, kmax, counts.ctypes.data,
                                          ctypes.byref(lat), self._err)
        if not ok:
            raise NativeError(self._lib.ngt_get_error_string(self._err).decode())
        m = int(counts.max()) if nq else 0
        return res["id"][:, :m].copy(), res["distance"][:, :m].copy(), counts, lat.value

    def close(self):
        if getattr(self, "_srv", None):
            self._lib.ngtgpu_server_destroy(self._srv)
            self._srv = None
        if getattr(self, "_err", None):
            self._lib.ngt_destroy_error_object(self._err)
            self._err = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
