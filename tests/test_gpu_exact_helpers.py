"""The FP64-pipe-free helpers of the plain path (fdf_exact.cuh: div_rn / div_by, d2f_rn, split_rn)
(and scale_down, mul_int, in_range) against the hardware instructions they replace, bit for bit, on the GPU: a small CUDA self-test
(tests/kernels/exact_selftest.cu) is compiled with the library's flags and run over seeded
operands from random bit patterns, the fast range, divisors near 1, extreme significands,
zeros, subnormals, infinities and NaNs."""
import ctypes
import os
import subprocess

import pytest

from fdf_gb300 import build as B

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def selftest(tmp_path_factory, require_gpu):
    out = str(tmp_path_factory.mktemp("exact") / "libexact_selftest.so")
    src = os.path.join(HERE, "kernels", "exact_selftest.cu")
    cmd = [B.nvcc()] + B.NVFLAGS + ["-I", B.CSRC, "-shared", src, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(out)
    lib.fdf_test_exact.argtypes = [ctypes.c_ulonglong, ctypes.c_longlong, ctypes.POINTER(ctypes.c_ulonglong)]
    lib.fdf_test_exact.restype = ctypes.c_int
    return lib


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_helpers_match_the_hardware_bit_for_bit(selftest, seed):
    out = (ctypes.c_ulonglong * 10)()
    n = 1 << 27
    assert selftest.fdf_test_exact(seed, n, out) == 0
    bad_a = ctypes.c_double.from_buffer_copy(ctypes.c_ulonglong(out[4])).value
    bad_b = ctypes.c_double.from_buffer_copy(ctypes.c_ulonglong(out[5])).value
    assert out[0] == 0, f"{out[0]} divisions differ from __ddiv_rn, first {bad_a!r} / {bad_b!r}"
    assert out[1] == 0, f"{out[1]} double -> float conversions differ"
    assert out[2] == 0, f"{out[2]} (hi, lo) splits differ"
    assert out[6] == 0, f"{out[6]} power-of-two scalings differ"
    assert out[7] == 0, f"{out[7]} integer-pipe products differ from __dmul_rn"
    assert out[8] == 0, f"{out[8]} integer-pipe range tests differ from the FP64 comparisons"
    assert out[9] == 0, f"{out[9]} bit predicates (lt0, eq0, is_nan, abs_lt, le_pos, add0, clamp01) differ"
    assert out[3] == n
