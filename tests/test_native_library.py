"""CPU-side checks of the native library: it builds, loads, exports every
function the public headers declare, and its index loader rejects damaged
index files with an error message (the loader runs before any CUDA call, so
this needs no GPU)."""
import ctypes
import gzip
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from golden_util import materialize

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "ngt_gb300", "libngtgpu.so")


def _have_nvcc():
    return shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        if not _have_nvcc():
            pytest.skip("libngtgpu.so not built and nvcc unavailable")
        from ngt_gb300.build import build_native
        build_native()
    return ctypes.CDLL(LIB)


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b((?:ngt|ngtgpu|ngtqg|qbg)_\w+)\s*\(", text, flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


def test_headers_declare_the_search_api():
    names = declared_functions()
    for must in ("ngt_open_index_as_read_only", "ngt_search_index_as_float", "ngt_linear_search_index_as_float",
                 "ngt_get_result", "ngtgpu_search_batch_float"):
        assert must in names


def test_library_exports_every_declared_function(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_library_is_built_for_sm_103a(lib):
    # the fatbin carries an sm_103a cubin; cuobjdump-free check through the ELF note nvcc writes
    data = open(LIB, "rb").read()
    assert b"sm_103a" in data or b"sm_103" in data


def _error_string(lib, fn, path):
    lib.ngt_create_error_object.restype = ctypes.c_void_p
    lib.ngt_get_error_string.restype = ctypes.c_char_p
    lib.ngt_get_error_string.argtypes = [ctypes.c_void_p]
    getattr(lib, fn).restype = ctypes.c_void_p
    getattr(lib, fn).argtypes = [ctypes.c_char_p, ctypes.c_void_p]
    err = lib.ngt_create_error_object()
    h = getattr(lib, fn)(path.encode(), ctypes.c_void_p(err))
    return h, lib.ngt_get_error_string(ctypes.c_void_p(err)).decode()


@pytest.mark.parametrize("damage", ["truncate_obj", "truncate_grp", "bad_edge", "missing_tre", "bad_prf"])
def test_loader_rejects_damaged_index(lib, tmp_path, damage):
    path, meta, _, _ = materialize("u8_l2", str(tmp_path))
    if damage == "truncate_obj":
        data = open(os.path.join(path, "obj"), "rb").read()
        open(os.path.join(path, "obj"), "wb").write(data[:-100])
    elif damage == "truncate_grp":
        data = open(os.path.join(path, "grp"), "rb").read()
        open(os.path.join(path, "grp"), "wb").write(data[: len(data) // 2])
    elif damage == "bad_edge":
        data = bytearray(open(os.path.join(path, "grp"), "rb").read())
        # first '+' record after the 8-byte count and the dummy '-': count, then (id, dist) pairs
        pos = 8 + 1 + 1 + 4
        data[pos:pos + 4] = np.uint32(10 ** 9).tobytes()
        open(os.path.join(path, "grp"), "wb").write(bytes(data))
    elif damage == "missing_tre":
        os.remove(os.path.join(path, "tre"))
    elif damage == "bad_prf":
        open(os.path.join(path, "prf"), "w").write("Dimension\tzero\n")
    h, msg = _error_string(lib, "ngt_open_index_as_read_only", path)
    assert h is None
    assert msg.startswith("Capi : ngt_open_index_as_read_only() : Error:")
    assert "CUDA" not in msg, msg


@pytest.mark.parametrize("damage", ["cosine", "no_scale", "zero_scale"])
def test_loader_rejects_unsupported_scalar_quantized_index(lib, tmp_path, damage):
    """QSUInteger-8B objects: L2 only, and a positive QuantizationScale is required."""
    path, meta, _, _ = materialize("qs8_l2", str(tmp_path))
    prf = open(os.path.join(path, "prf")).read().splitlines()
    if damage == "cosine":
        prf = [l if not l.startswith("DistanceType\t") else "DistanceType\tCosine" for l in prf]
    elif damage == "no_scale":
        prf = [l for l in prf if not l.startswith("QuantizationScale\t")]
    else:
        prf = [l if not l.startswith("QuantizationScale\t") else "QuantizationScale\t0" for l in prf]
    open(os.path.join(path, "prf"), "w").write("\n".join(prf) + "\n")
    h, msg = _error_string(lib, "ngt_open_index_as_read_only", path)
    assert h is None
    assert "QSUInteger-8B" in msg, msg


def test_null_arguments_return_false_with_message(lib):
    lib.ngt_create_error_object.restype = ctypes.c_void_p
    lib.ngt_get_error_string.restype = ctypes.c_char_p
    lib.ngt_get_error_string.argtypes = [ctypes.c_void_p]
    lib.ngt_search_index_as_float.restype = ctypes.c_bool
    lib.ngt_search_index_as_float.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_size_t,
                                              ctypes.c_float, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p]
    err = ctypes.c_void_p(lib.ngt_create_error_object())
    ok = lib.ngt_search_index_as_float(None, None, 0, 10, 0.1, -1.0, None, err)
    assert not ok
    assert "parametor error" in lib.ngt_get_error_string(err).decode()


def test_tensor_core_search_rejects_null_arguments(lib):
    """The tensor-core exhaustive search entry points check their handles and
    buffers before any device work."""
    lib.ngt_create_error_object.restype = ctypes.c_void_p
    lib.ngt_get_error_string.restype = ctypes.c_char_p
    lib.ngt_get_error_string.argtypes = [ctypes.c_void_p]
    vp, sz = ctypes.c_void_p, ctypes.c_size_t
    calls = {
        "ngtgpu_linear_search_tc_float": ([vp, vp, sz, ctypes.c_int32, sz, sz, vp, sz, vp, vp, vp],
                                          (None, None, 4, 8, 10, 0, None, 10, None, None)),
        "ngtgpu_linear_search_tc_device": ([vp, vp, sz, sz, sz, vp, sz, vp, vp, vp, vp],
                                           (None, None, 4, 10, 0, None, 10, None, None, None)),
        "ngtgpu_tc_scores_device": ([vp, vp, sz, vp, sz, vp, vp], (None, None, 4, None, 100, None)),
        "ngtgpu_set_tc_first_rows": ([vp, sz, vp], (None, 0)),
        "ngtgpu_tc_phase_times": ([vp, vp, vp], (None, None)),
        "ngtgpu_set_tc_graphs": ([vp, ctypes.c_int32, vp], (None, 1)),
        "ngtgpu_linear_search_tc_ex": ([vp, vp, sz, sz, sz, ctypes.c_uint32, ctypes.c_uint32, vp, sz, vp, vp, vp, vp],
                                       (None, None, 4, 10, 0, 0, 2, None, 10, None, None, None)),
    }
    for name, (argtypes, args) in calls.items():
        fn = getattr(lib, name)
        fn.argtypes = argtypes
        fn.restype = ctypes.c_bool
        err = ctypes.c_void_p(lib.ngt_create_error_object())
        assert not fn(*args, err), name
        assert "parametor error" in lib.ngt_get_error_string(err).decode(), name


@pytest.mark.parametrize("damage", ["truncate_qg_grp", "missing_qr", "short_codebook", "bad_qg_edge", "no_qg",
                                    "wrong_metric"])
def test_qg_loader_rejects_damaged_quantized_graph(lib, tmp_path, damage):
    path, meta, _, _ = materialize("qg_f32_l2_d32", str(tmp_path))
    qg = os.path.join(path, "qg")
    if damage == "truncate_qg_grp":
        data = open(os.path.join(qg, "grp"), "rb").read()
        open(os.path.join(qg, "grp"), "wb").write(data[: len(data) - 7])
    elif damage == "missing_qr":
        os.remove(os.path.join(qg, "qr"))
    elif damage == "short_codebook":
        data = open(os.path.join(qg, "local-3", "obj"), "rb").read()
        rec = 1 + 4                                   # '+' and one float (one dimension per subspace)
        out = np.uint64(16).tobytes() + data[8:8 + 1 + 15 * rec]
        open(os.path.join(qg, "local-3", "obj"), "wb").write(out)
    elif damage == "bad_qg_edge":
        data = bytearray(open(os.path.join(qg, "grp"), "rb").read())
        # node 0 (no edges): sid, count 0; node 1: sid, count, then its first id
        pos = 16 + 8 + 4 + 4
        data[pos:pos + 4] = np.uint32(10 ** 9).tobytes()
        open(os.path.join(qg, "grp"), "wb").write(bytes(data))
    elif damage == "no_qg":
        shutil.rmtree(qg)
    elif damage == "wrong_metric":
        prf = open(os.path.join(path, "prf")).read().replace("DistanceType\tL2", "DistanceType\tL1")
        open(os.path.join(path, "prf"), "w").write(prf)
    h, msg = _error_string(lib, "ngtqg_open_index", path)
    assert h is None
    assert msg.startswith("Capi : ngtqg_open_index() : Error:"), msg
    assert "CUDA" not in msg, msg


@pytest.mark.parametrize("damage", ["missing_rqcb", "bad_sid", "truncate_grp", "no_global"])
def test_qbg_loader_rejects_damaged_index(lib, tmp_path, damage):
    from golden_util import fixture_names
    path, meta, _, _ = materialize(fixture_names("qbg")[0], str(tmp_path))
    if damage == "missing_rqcb":
        os.remove(os.path.join(path, "rqcb"))
    elif damage == "bad_sid":
        data = bytearray(open(os.path.join(path, "grp"), "rb").read())
        pos = 16 + 8                                  # node 1's subspace id (node 0 is empty)
        data[pos:pos + 4] = np.uint32(10 ** 6).tobytes()
        open(os.path.join(path, "grp"), "wb").write(bytes(data))
    elif damage == "truncate_grp":
        data = open(os.path.join(path, "grp"), "rb").read()
        open(os.path.join(path, "grp"), "wb").write(data[: len(data) - 5])
    elif damage == "no_global":
        shutil.rmtree(os.path.join(path, "global"))
    lib.qbg_open_index.restype = ctypes.c_void_p
    lib.qbg_open_index.argtypes = [ctypes.c_char_p, ctypes.c_bool, ctypes.c_void_p]
    lib.ngt_create_error_object.restype = ctypes.c_void_p
    lib.ngt_get_error_string.restype = ctypes.c_char_p
    lib.ngt_get_error_string.argtypes = [ctypes.c_void_p]
    err = lib.ngt_create_error_object()
    h = lib.qbg_open_index(path.encode(), True, ctypes.c_void_p(err))
    msg = lib.ngt_get_error_string(ctypes.c_void_p(err)).decode()
    assert h is None
    assert msg.startswith("Capi : qbg_open_index() : Error:"), msg
    assert "CUDA" not in msg, msg
