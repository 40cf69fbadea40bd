"""Mixed-radix addressing of folded mode groups (group_offset in
muscle.jl_gb300/csrc/mgb_internal.h), compiled for the host with g++ and
checked against a direct decomposition, across the 32-bit fast path and the
64-bit one (indices and extents beyond 2^31)."""
import ctypes
import os
import random
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "muscle.jl_gb300", "csrc")
INCLUDE = os.path.join(ROOT, "include")

SHIM = r'''
#include "mgb_internal.h"
extern "C" long long offset_of(int n, const long long *ext, const long long *str, long long idx) {
    mgb::ModeGroup g;
    g.n = n;
    for (int i = 0; i < n; ++i) {
        g.ext[i] = ext[i];
        g.str[0][i] = 0;
        g.str[1][i] = str[i];
        g.str[2][i] = 0;
    }
    return mgb::group_offset(g, 1, idx);
}
'''


def _cuda_include():
    for base in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if base and os.path.exists(os.path.join(base, "include", "cuda_runtime.h")):
            return os.path.join(base, "include")
    return None


@pytest.fixture(scope="module")
def offset_of(tmp_path_factory):
    gxx, inc = shutil.which("g++"), _cuda_include()
    if gxx is None or inc is None:
        pytest.skip("g++ or the CUDA headers are not available")
    d = tmp_path_factory.mktemp("gofs")
    src, so = d / "shim.cpp", d / "libgofs.so"
    src.write_text(SHIM)
    subprocess.run([gxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I" + inc, "-I" + CSRC, "-I" + INCLUDE,
                    str(src), "-o", str(so)], check=True)
    lib = ctypes.CDLL(str(so))
    lib.offset_of.restype = ctypes.c_longlong
    lib.offset_of.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong),
                              ctypes.c_longlong]

    def f(ext, st, idx):
        n = len(ext)
        E = (ctypes.c_longlong * max(n, 1))(*ext)
        S = (ctypes.c_longlong * max(n, 1))(*st)
        return lib.offset_of(n, E, S, idx)

    return f


def direct(ext, st, idx):
    off = 0
    for e, s in zip(ext, st):
        off += (idx % e) * s
        idx //= e
    return off


def test_small_and_large_groups(offset_of):
    rng = random.Random(11)
    cases = [([], []), ([7], [3]), ([2, 8, 8, 8], [1, 2, 16, 128]), ([5, 3, 4], [60, 1, 3])]
    # extents whose product passes 2^31, and one extent above 2^31
    cases += [([1 << 16, 1 << 16, 3], [1, 1 << 16, 1 << 32]), ([3, (1 << 31) + 11], [1 << 33, 3])]
    for ext, st in cases:
        size = 1
        for e in ext:
            size *= e
        idxs = {0, size - 1} | {rng.randrange(size) for _ in range(300)}
        idxs |= {i for i in ((1 << 31) - 1, 1 << 31, (1 << 31) + 1) if i < size}
        for i in idxs:
            assert offset_of(ext, st, i) == direct(ext, st, i), (ext, st, i)
