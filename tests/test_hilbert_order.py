"""CPU checks of the Hilbert face ordering (csrc/hilbert.cpp) that numbers
the faces internally and so decides which side owns each interior edge of
the mixed path: the order is the stable sort of the faces by Hilbert key
(ties in reference order), the same for any thread count."""
from __future__ import annotations

import ctypes
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
CSRC = REPO / "muscl-scheme-on-spherical-mesh-wip_gb300" / "csrc"


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    out = tmp_path_factory.mktemp("hilbert") / "libhilbert.so"
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-fopenmp", f"-I{CSRC}",
           str(REPO / "tests" / "cpp" / "hilbert_order.cpp"), str(CSRC / "hilbert.cpp"), "-o", str(out)]
    subprocess.run(cmd, check=True, capture_output=True)
    lib = ctypes.CDLL(str(out))
    lib.ho_key.restype = ctypes.c_uint64
    lib.ho_key.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int]
    return lib


def _order(lib, xyz, threads):
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    out = np.empty(len(xyz), np.int32)
    lib.ho_order(xyz.ctypes.data_as(ctypes.c_void_p), ctypes.c_int(len(xyz)), ctypes.c_int(threads),
                 out.ctypes.data_as(ctypes.c_void_p))
    return out


@pytest.mark.parametrize("n", [1, 2, 7, 1000, 50000])
def test_stable_sort_by_key_any_thread_count(lib, n):
    rng = np.random.default_rng(n)
    xyz = rng.standard_normal((n, 3))
    # repeated points give equal keys: ties must stay in input order
    xyz[5::10] = xyz[0:len(xyz[5::10]) * 10:10][: len(xyz[5::10])]
    # the normalisation hilbert_order applies: sqrt((x x + y y) + z z)
    nrm = np.sqrt((xyz[:, 0] * xyz[:, 0] + xyz[:, 1] * xyz[:, 1]) + xyz[:, 2] * xyz[:, 2])
    r = xyz / nrm[:, None]
    keys = np.array([lib.ho_key(float(a), float(b), float(c), 21) for a, b, c in r], dtype=np.uint64)
    expected = np.argsort(keys, kind="stable").astype(np.int32)
    for threads in (1, 2, 4):
        assert np.array_equal(_order(lib, xyz, threads), expected), threads
