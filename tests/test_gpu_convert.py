"""The refinement converts FP64 matrices to FP32 on the integer pipes
(magma_gb300/csrc/convert.cuh).  It must agree bit for bit with CUDA's own
round-to-nearest-even conversion (__double2float_rn) -- checked here on 2^26
inputs: random bit patterns and values placed at float rounding boundaries,
exact ties and the float subnormal range."""
import ctypes as C
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu


def test_integer_d2f_matches_cuda(cuda):
    lib = C.CDLL(str(Path(__file__).resolve().parent.parent / "magma_gb300" / "libmlu_probe.so"))
    lib.mlu_check_d2f.restype = C.c_longlong
    lib.mlu_check_d2f.argtypes = [C.c_longlong, C.c_ulonglong]
    for seed in (1, 2):
        assert lib.mlu_check_d2f(1 << 26, seed) == 0
