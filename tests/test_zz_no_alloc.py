"""The search entry point that allocates no device memory.

ngtgpu_search_exact_noalloc exists for callers that cannot call cudaMalloc
while they search (hosts that own all device memory, allocator-free serving
paths).  It runs the exact-order kernel with its scratch carved from a fixed
device array, so its results must equal the regular entry point's
(ngtgpu_search_batch_device, exact kernel) -- bit for bit on this
integer-valued index -- and keep doing so on consecutive calls that reuse the
array.  This file is collected last so that a failure here leaves every other
test already run.
"""
import ctypes

import numpy as np
import pytest

from golden_util import materialize

pytestmark = pytest.mark.gpu


def _cudart():
    """The CUDA runtime this process already loaded (for the memory queries)."""
    for line in open("/proc/self/maps"):
        path = line.split()[-1] if line.strip() else ""
        if "libcudart.so" in path:
            return ctypes.CDLL(path)
    raise RuntimeError("libcudart is not loaded")


def _device_memory_state(rt):
    """(free device bytes, default pool reserved bytes, default pool used bytes)."""
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    assert rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    pool = ctypes.c_void_p()
    dev = ctypes.c_int()
    assert rt.cudaGetDevice(ctypes.byref(dev)) == 0
    assert rt.cudaDeviceGetDefaultMemPool(ctypes.byref(pool), dev) == 0
    reserved, used = ctypes.c_uint64(), ctypes.c_uint64()
    assert rt.cudaMemPoolGetAttribute(pool, 5, ctypes.byref(reserved)) == 0      # ReservedMemCurrent
    assert rt.cudaMemPoolGetAttribute(pool, 7, ctypes.byref(used)) == 0          # UsedMemCurrent
    return free.value, reserved.value, used.value


def _noalloc(lib):
    fn = lib.ngtgpu_search_exact_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                   ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p]
    fn.restype = ctypes.c_bool
    return fn


def test_noalloc_equals_regular_entry_point_on_consecutive_calls(tmp_path):
    import torch
    from ngt_gb300 import Index
    from ngt_gb300.base import KERNEL_EXACT, QUERY_STATS_DTYPE
    path, meta, queries, golden = materialize("c1_f32_l2", str(tmp_path))
    nq, k = 300, 10
    with Index(path, read_only=True) as ix:
        ix.batch_search(queries[:4], k=k, epsilon=0.1)          # builds the seed table for k
        rows = torch.from_numpy(ix.convert_queries(queries[:nq])).cuda()
        params, nparams = ix.make_params(k, 0.1)
        sw = QUERY_STATS_DTYPE.itemsize // 4

        def buffers():
            return (torch.zeros((nq, k, 2), dtype=torch.int32, device="cuda"),
                    torch.zeros(nq, dtype=torch.int32, device="cuda"),
                    torch.zeros((nq, sw), dtype=torch.int32, device="cuda"))

        ra, ca, sa = buffers()
        ix.search_device(rows.data_ptr(), nq, params, nparams, ra.data_ptr(), k, ca.data_ptr(), sa.data_ptr(),
                         kernel=KERNEL_EXACT)
        torch.cuda.synchronize()
        fn = _noalloc(ix._lib)
        rt = _cudart()
        for call in range(2):
            rb, cb, sb = buffers()
            torch.cuda.synchronize()
            before = _device_memory_state(rt)
            ok = fn(ix._index, rows.data_ptr(), nq, params, nparams, rb.data_ptr(), k, cb.data_ptr(), sb.data_ptr(),
                    None, ix._err)
            assert ok, ix._lib.ngt_get_error_string(ix._err)
            torch.cuda.synchronize()
            # nothing reserved on the device by the call: free memory and the default
            # pool unchanged (the fixed scratch was reserved when the index opened)
            assert _device_memory_state(rt) == before, call
            assert torch.equal(ca, cb)
            assert torch.equal(ra, rb)          # ids and distance bits
            assert torch.equal(sa, sb)          # identical search work
        # and both equal the reference's golden results
        ids = ra[:, :, 0].cpu().numpy().view(np.uint32)
        assert np.array_equal(ids, golden["ids_0"][:nq])


def test_noalloc_rejects_requests_beyond_its_scratch(tmp_path):
    import torch
    from ngt_gb300 import Index
    path, meta, queries, _ = materialize("c1_f32_l2", str(tmp_path))
    with Index(path, read_only=True) as ix:
        ix.batch_search(queries[:4], k=10, epsilon=0.1)
        dummy = torch.zeros(16, dtype=torch.int32, device="cuda")
        params, nparams = ix.make_params(10, 0.1)
        fn = _noalloc(ix._lib)
        nq = 2_000_000                          # parameter blocks alone exceed the 32 MiB scratch
        ok = fn(ix._index, dummy.data_ptr(), nq, params, nparams, dummy.data_ptr(), 10, dummy.data_ptr(),
                dummy.data_ptr(), None, ix._err)
        assert not ok
        msg = ix._lib.ngt_get_error_string(ix._err).decode()
        assert "scratch" in msg and "fewer queries" in msg
        ix._lib.ngt_clear_error_string(ix._err)
        # a result size without a prepared seed table is refused, not built
        params2, n2 = ix.make_params(3, 0.1)
        ok = fn(ix._index, dummy.data_ptr(), 1, params2, n2, dummy.data_ptr(), 3, dummy.data_ptr(), dummy.data_ptr(),
                None, ix._err)
        assert not ok
        assert "seed table" in ix._lib.ngt_get_error_string(ix._err).decode()
