"""Pins the oracle's query rotation (Rotation::mul, lib/NGT/NGTQ/Quantizer.h:117-160)
to the BLAS sgemv the reference calls for it.

The reference rotates QG/QBG queries with BLAS sgemv; its x86-64 build here links
scipy's OpenBLAS.  The oracle (and the GPU kernels, which follow the same order)
restate that sgemv's summation order; this test checks the restatement against the
library itself, bit for bit, at every multiple of 16 up to 768 (QG/QBG
pseudo-dimensions are multiples of 16, lib/NGT/NGTQ/QuantizedGraph.h:640-657).
"""
import ctypes
import platform

import numpy as np
import pytest

import oracle


@pytest.mark.skipif(platform.machine() not in ("x86_64", "AMD64"),
                    reason="the restated order is the x86-64 OpenBLAS kernel's")
@pytest.mark.parametrize("d", [16, 32, 48, 64, 80, 96, 112, 128, 144, 192, 256, 384, 512, 768])
def test_rotation_equals_linked_sgemv(d):
    blas = pytest.importorskip("scipy.linalg.blas")
    lib = ctypes.CDLL(oracle.build())
    lib.oracle_rotate.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
    rng = np.random.default_rng(d)
    for _ in range(20):
        R = np.ascontiguousarray(rng.standard_normal((d, d)), np.float32)      # element [p * d + c]
        x = np.ascontiguousarray(rng.standard_normal(d), np.float32)
        y = np.zeros(d, np.float32)
        lib.oracle_rotate(R.ctypes.data, x.ctypes.data, y.ctypes.data, d)
        # column-major A(c, p) = R[p * d + c], y = A x: what sgemv('N') computes on R's buffer
        want = blas.sgemv(1.0, np.asfortranarray(R.T), x)
        assert np.array_equal(y.view(np.uint32), np.asarray(want, np.float32).view(np.uint32)), d
