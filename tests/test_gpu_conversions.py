"""The integer-pipe binary32 <-> binary64 conversions (f2d_bits, d2f_bits in
device_math.cuh) give the same bits as the hardware conversion and as IEEE
754 round-to-nearest-even (numpy's astype), on every class of input."""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

from mgcfd import _build

pytestmark = pytest.mark.gpu
HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def conv():
    out = HERE / "_build" / "libconv_check.so"
    out.parent.mkdir(exist_ok=True)
    src = HERE / "native" / "conv_check.cu"
    subprocess.run([_build._nvcc(), *_build.ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
                    f"-I{_build.CSRC}", str(src), "-o", str(out)], check=True, capture_output=True)
    lib = C.CDLL(str(out))
    lib.conv_check.restype = C.c_int
    return lib


def run(lib, d, f):
    d = np.ascontiguousarray(d, dtype=np.float64)
    f = np.ascontiguousarray(f, dtype=np.float32)
    o = [np.empty(len(d), np.float32), np.empty(len(d), np.float32), np.empty(len(f)), np.empty(len(f))]
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    assert lib.conv_check(C.c_int64(len(d)), p(d), p(o[0]), p(o[1]), C.c_int64(len(f)), p(f), p(o[2]), p(o[3])) == 0
    return o


def same_bits(a, b):
    nan = np.isnan(a) & np.isnan(b)
    return np.where(nan, True, a.view(np.uint32 if a.dtype == np.float32 else np.uint64)
                    == b.view(np.uint32 if b.dtype == np.float32 else np.uint64))


def test_double_to_float_and_back(conv):
    rng = np.random.default_rng(5)
    rand_bits = (rng.integers(0, 2 ** 63, 400_000, dtype=np.int64).astype(np.uint64)
                 | (rng.integers(0, 2, 400_000).astype(np.uint64) << np.uint64(63))).view(np.float64)
    # values in binary32's range, and exact halfway cases between floats
    f_vals = rng.integers(0, 0x7f800000, 200_000, dtype=np.int64).astype(np.uint32).view(np.float32)
    fd = f_vals.astype(np.float64)
    half = np.nextafter(f_vals, np.float32(np.inf)).astype(np.float64)
    mid = fd + (half - fd) / 2
    edges = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, -1.0, 3.4028234663852886e38, 3.4028235677973366e38,
                      3.4028235677973362e38, 3.4028235677973370e38, 1e39, 1.1754943508222875e-38,
                      1.1754942807573643e-38, 1.401298464324817e-45, 7.006492321624085e-46, 7.006492321624087e-46,
                      2.1019476964872256e-45, 1e-46, 5e-324, -5e-324, 2.2250738585072014e-308])
    sub = (rng.integers(1, 2 ** 23, 100_000).astype(np.float64) + rng.choice([0.0, 0.25, 0.5, 0.75], 100_000)) \
        * 1.401298464324817e-45
    d = np.concatenate([rand_bits, fd, mid, np.nextafter(mid, np.inf), np.nextafter(mid, -np.inf), edges, sub, -sub])
    f = np.concatenate([f_vals, -f_vals, np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-45, -1e-45, 1e-40],
                                                   np.float32),
                        rng.integers(1, 2 ** 23, 100_000, dtype=np.int64).astype(np.uint32).view(np.float32)])
    d2f_hw, d2f_int, f2d_hw, f2d_int = run(conv, d, f)
    with np.errstate(over="ignore"):
        want = d.astype(np.float32)
    assert same_bits(d2f_int, d2f_hw).all()
    assert same_bits(d2f_int, want).all()
    assert same_bits(f2d_int, f2d_hw).all()
    assert same_bits(f2d_int, f.astype(np.float64)).all()
