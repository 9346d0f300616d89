"""The solver's shared-reciprocal division (diomedes_gb300/csrc/div_rn.cuh)
against IEEE round-to-nearest division, bit for bit.

Inside its range the correction step scales exactly with the exponents of a
and b, so the significand pairs in [1, 2) decide it: the sweep compares every
a significand with a strided set of b significands (every b with
DIO_FULL_DIVISION_SWEEP=1, about a minute); random full-range pairs and the
special values (zeros, subnormals, infinities, NaN, extreme exponents) are
compared with numpy's float32 division."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "diomedes_gb300", "csrc")


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = str(tmp_path_factory.mktemp("div") / "libdivcheck.so")
    subprocess.check_call([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-shared",
                           "-Xcompiler", "-fPIC", "-I", CSRC, os.path.join(HERE, "division_check.cu"), "-o", out])
    L = ctypes.CDLL(out)
    L.div_sweep.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                            ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_uint32)]
    L.div_pairs.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p]
    return L


def test_every_a_significand_against_b_significands(harness):
    stride = 1 if os.environ.get("DIO_FULL_DIVISION_SWEEP") == "1" else 61
    count = ((1 << 23) + stride - 1) // stride
    bad = ctypes.c_ulonglong(0)
    wit = (ctypes.c_uint32 * 3)()
    assert harness.div_sweep(0, count, stride, ctypes.byref(bad), wit) == 0
    a = np.array([wit[1]], np.uint32).view(np.float32)[0]
    b = np.array([wit[2]], np.uint32).view(np.float32)[0]
    assert bad.value == 0, f"{bad.value} mismatches, first a={a!r} b={b!r}"


def _pairs(harness, a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    out = np.zeros_like(a)
    assert harness.div_pairs(a.ctypes.data, b.ctypes.data, len(a), out.ctypes.data) == 0
    return out


def _same(got, want):
    both_nan = np.isnan(got) & np.isnan(want)
    return (got.view(np.uint32) == want.view(np.uint32)) | both_nan


def test_random_full_range_and_special_pairs(harness):
    rng = np.random.default_rng(7)
    n = 1 << 22
    # random bit patterns (every exponent, both signs, subnormals, specials)
    a = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32).view(np.float32)
    b = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32).view(np.float32)
    # values like the solver's pivots and entries: moderate exponents
    m = rng.uniform(-1, 1, n).astype(np.float32) * np.exp2(rng.integers(-40, 40, n)).astype(np.float32)
    d = rng.uniform(0.1, 10, n).astype(np.float32) * np.exp2(rng.integers(-40, 40, n)).astype(np.float32)
    special = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, 1e-45, -1e-45, 1.17549435e-38,
                        2.0 ** -96, 2.0 ** 96, 2.0 ** -97, 2.0 ** 97, 3.4028235e38, 0.5, 3.0], np.float32)
    sa, sb = np.meshgrid(special, special)
    A = np.concatenate([a, m, sa.ravel()])
    B = np.concatenate([b, d, sb.ravel()])
    with np.errstate(all="ignore"):
        want = A / B
    got = _pairs(harness, A, B)
    ok = _same(got, want)
    bad = np.flatnonzero(~ok)
    assert bad.size == 0, f"{bad.size} mismatches, e.g. {A[bad[0]]!r} / {B[bad[0]]!r}: {got[bad[0]]!r} vs {want[bad[0]]!r}"
