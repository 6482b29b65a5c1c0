"""Builds the native library ngt_gb300/libngtgpu.so with nvcc for sm_103a.

Every translation unit is compiled in parallel into ngt_gb300/_build/ and
linked into one shared library that exports the C ABI declared in
include/ngt_capi.h and include/ngtgpu.h.  Objects are rebuilt only when a
source or header is newer than them.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libngtgpu.so")
LOOP = os.path.join(PKG, "capi_loop")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + CSRC, "-I" + os.path.join(ROOT, "include")]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libngtgpu.so")


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers_mtime() -> float:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".inc"))]
    hs += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    return max(os.path.getmtime(h) for h in hs)


def build_native(verbose: bool = False, jobs: int | None = None) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    hdr = _headers_mtime()
    cmds = []
    objs = []
    for src in _sources():
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if os.path.exists(o) and os.path.getmtime(o) >= max(os.path.getmtime(s), hdr):
            continue
        lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
        cmds.append([nvcc] + NVCC_FLAGS + lang + ["-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        return r.stderr

    with ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        for err in ex.map(run, cmds):
            if verbose and err:
                print(err, flush=True)
    if cmds or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    # the native multi-threaded caller of the C API (benchmark of the drop-in path)
    src = os.path.join(PKG, "capi_loop.c")
    if not os.path.exists(LOOP) or os.path.getmtime(LOOP) < max(os.path.getmtime(src), os.path.getmtime(LIB)):
        cc = shutil.which("gcc") or shutil.which("cc")
        if cc is None:
            raise RuntimeError("no C compiler for capi_loop.c")
        run([cc, "-O2", "-std=gnu11", "-I" + os.path.join(ROOT, "include"), src, "-o", LOOP, "-L" + PKG,
             "-lngtgpu", "-lpthread", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build_native(verbose=True))
