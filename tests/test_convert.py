"""The integer-only float conversions of the data-movement kernels
(vmps_gb300/csrc/convert.hpp) against the CPU's IEEE conversions: compiled for
the host with g++ and run over edge cases and random bit patterns."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = r"""
#include "convert.hpp"
extern "C" void to_f32(const double* x, float* y, long n) { for (long i = 0; i < n; ++i) y[i] = vmps::f64_to_f32_rn(x[i]); }
extern "C" void to_f64(const float* x, double* y, long n) { for (long i = 0; i < n; ++i) y[i] = vmps::f32_to_f64(x[i]); }
"""


@pytest.fixture(scope="module")
def conv(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("conv")
    src = d / "conv.cpp"
    src.write_text(SRC)
    so = d / "libconv.so"
    subprocess.run(["g++", "-O2", "-shared", "-fPIC", "-std=c++17", "-I", os.path.join(ROOT, "vmps_gb300", "csrc"),
                    str(src), "-o", str(so)], check=True)
    lib = C.CDLL(str(so))
    lib.to_f32.argtypes = [C.c_void_p, C.c_void_p, C.c_long]
    lib.to_f64.argtypes = [C.c_void_p, C.c_void_p, C.c_long]
    return lib


def _to_f32(lib, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty(x.size, dtype=np.float32)
    lib.to_f32(x.ctypes.data, y.ctypes.data, x.size)
    return y


def _to_f64(lib, x):
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty(x.size, dtype=np.float64)
    lib.to_f64(x.ctypes.data, y.ctypes.data, x.size)
    return y


def _same_bits32(a, b):
    a, b = a.view(np.uint32), b.view(np.uint32)
    nan = np.isnan(a.view(np.float32)) & np.isnan(b.view(np.float32))
    return np.all((a == b) | nan)


def test_f64_to_f32_edge_cases(conv):
    f32 = np.finfo(np.float32)
    tiny_sub = np.float64(2.0 ** -149)
    xs = [0.0, -0.0, 1.0, -1.0, 1.5, np.pi, -np.e, 1e-40, -1e-45, 1e-46, 1e-300, 5e-324, -5e-324,
          float(f32.max), float(f32.max) * (1 + 2 ** -25), float(f32.max) * (1 + 2 ** -23), 3.5e38, 1e300,
          float(f32.tiny), float(f32.tiny) * (1 - 2 ** -30), tiny_sub, tiny_sub * 0.5, tiny_sub * 0.5000001,
          tiny_sub * 1.5, tiny_sub * 2.5, np.inf, -np.inf, np.nan,
          1 + 2 ** -24, 1 + 3 * 2 ** -24, 1 + 2 ** -24 + 2 ** -50, 2 ** 127 * (2 - 2 ** -24)]
    x = np.array(xs, dtype=np.float64)
    with np.errstate(over="ignore"):
        ref = x.astype(np.float32)
    assert _same_bits32(_to_f32(conv, x), ref)


def test_f64_to_f32_random_bits(conv):
    rng = np.random.default_rng(0)
    bits = rng.integers(0, 2 ** 63, size=400000, dtype=np.uint64) | (rng.integers(0, 2, 400000, dtype=np.uint64) << 63)
    x = bits.view(np.float64)
    # concentrate half of them around the float range, where rounding happens
    e = rng.integers(1023 - 160, 1023 + 130, size=200000).astype(np.uint64)
    x[:200000] = ((bits[:200000] & np.uint64(0x800FFFFFFFFFFFFF)) | (e << np.uint64(52))).view(np.float64)
    with np.errstate(over="ignore", invalid="ignore"):
        ref = x.astype(np.float32)
    assert _same_bits32(_to_f32(conv, x), ref)


def test_f32_to_f64_exact(conv):
    rng = np.random.default_rng(1)
    bits = rng.integers(0, 2 ** 32, size=400000, dtype=np.uint64).astype(np.uint32)
    x = bits.view(np.float32)
    edge = np.array([0.0, -0.0, 1e-45, -1e-45, 1.17e-38, 3.4e38, np.inf, -np.inf, 1.0, -2.5], dtype=np.float32)
    x = np.concatenate([x, edge, (np.arange(1, 5000, dtype=np.uint32)).view(np.float32)])
    got = _to_f64(conv, x)
    with np.errstate(invalid="ignore"):
        ref = x.astype(np.float64)
    ok = (got.view(np.uint64) == ref.view(np.uint64)) | (np.isnan(got) & np.isnan(ref))
    assert np.all(ok)
