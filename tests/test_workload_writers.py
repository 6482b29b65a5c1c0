"""CPU tests of the benchmark's index writers and helpers: the scalar-quantized
index writer codes objects exactly as the oracle (pinned to the reference) codes
queries, its files read back through the oracle's independent reader, and the
tie-aware recall counts what it should."""

import numpy as np

import oracle


def test_symmetric_quantization_matches_the_oracle():
    import ctypes
    from ngt_gb300 import graph_build
    L = ctypes.CDLL(oracle.build())
    L.oracle_prepare_qsint8.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                        ctypes.c_float, ctypes.c_int, ctypes.c_void_p]
    rng = np.random.default_rng(7)
    x = (rng.standard_normal((300, 32)) * 3).astype(np.float32)
    x[0, :4] = [0.5, -0.5, 2.5, -2.5]                       # halves: rounding away from zero
    for scale in (float(np.abs(x).max()), 127.5, 3.3):
        ours = graph_build.quantize_symmetric(x, scale)
        ref = np.zeros((len(x), 32), np.int8)
        L.oracle_prepare_qsint8(32, x.ctypes.data, len(x), 32, ctypes.c_float(scale), 0, ref.ctypes.data)
        assert np.array_equal(ours, ref), scale


def test_qsint8_index_reads_back(tmp_path):
    from ngt_gb300 import graph_build
    rng = np.random.default_rng(8)
    x = rng.integers(0, 256, size=(50, 16)).astype(np.float32)
    n = len(x)
    # a small float graph-only index: node i (1-based) linked to its two successors
    offsets = np.zeros(n + 2, np.int64)
    edges = []
    for i in range(1, n + 1):
        nb = [((i % n) + 1), (((i + 1) % n) + 1)]
        edges += nb
        offsets[i + 1] = offsets[i] + len(nb)
    edges = np.array(edges, np.uint32)
    fpath, qpath = str(tmp_path / "f"), str(tmp_path / "q")
    graph_build.write_index(fpath, x, offsets, edges, np.zeros(len(edges), np.float32))
    scale = graph_build.write_qsint8_index(qpath, fpath, x, log=lambda *a: None)
    assert scale == 255.0
    f = oracle.IndexFiles(qpath)
    assert f.prop["ObjectType"] == "QSUInteger-8B" and float(f.prop["QuantizationScale"]) == 255.0
    assert np.array_equal(f.objects[1:, :16], graph_build.quantize_symmetric(x, scale))
    g = oracle.IndexFiles(fpath)
    assert np.array_equal(f.offsets, g.offsets) and np.array_equal(f.edges, g.edges)


def test_tie_aware_recall():
    import bench
    base = np.array([[0, 0], [1, 0], [0, 1], [3, 3]], np.float32)
    queries = np.array([[0, 0]], np.float32)
    kth = np.array([1.0])                        # the 2nd smallest squared distance
    # ids 1-based: object 3 ties with object 2 at distance 1, object 4 is beyond
    assert bench.recall(base, queries, np.array([[1, 3]], np.uint32), np.array([2]), kth, 2) == 1.0
    assert bench.recall(base, queries, np.array([[1, 4]], np.uint32), np.array([2]), kth, 2) == 0.5
    assert bench.recall(base, queries, np.array([[1, 0]], np.uint32), np.array([1]), kth, 2) == 0.5


def test_clock_sampler_keeps_the_samples_of_its_region(tmp_path, monkeypatch):
    """A stand-in nvidia-smi prints a sample every period with its own timestamp; the
    summary counts the samples inside the region and reports an active reason."""
    import os
    import time
    import bench
    fake = tmp_path / "nvidia-smi"
    fake.write_text(
        "#!" + __import__("sys").executable + "\n"
        "import datetime, sys, time\n"
        "period = int(sys.argv[sys.argv.index('-lms') + 1]) / 1000.0\n"
        "while True:\n"
        "    t = datetime.datetime.now().strftime('%Y/%m/%d %H:%M:%S.%f')[:-3]\n"
        "    print(t + ', 0, 1965, 2070, 900.1, 0x4, Not Active, Not Active, Not Active, Active', flush=True)\n"
        "    time.sleep(period)\n")
    fake.chmod(0o755)
    monkeypatch.setenv("PATH", str(tmp_path) + os.pathsep + os.environ["PATH"])
    with bench.ClockSampler(0, period_ms=20) as c:
        time.sleep(0.3)
    s = c.summary()
    assert s["sm_mhz"] == 1965.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]
    assert 5 <= s["samples_in_region"] <= 20 and s["samples_in_region"] < len(c.rows)   # lead-in dropped
