"""particle2grid!'s weight inv(sqrt(ss)^2) evaluated on the integer pipe
(csrc/jp_weight.cuh) against CUDA's correctly rounded double sqrt, multiply
and reciprocal, bit for bit, on billions of seeded inputs covering the whole
double range and its edge families (the parity tests against the oracle
cover the weights particle2grid! actually meets)."""
import ctypes

import pytest

from _harness import jp

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 0x5EED])
def test_integer_weight_matches_cuda_chain(seed):
    lib = jp._native.load()
    bad = ctypes.c_int64(-1)
    first = ctypes.c_uint64(0)
    n = 1 << 32
    assert lib.jp_selftest_weight(seed, n, ctypes.byref(bad), ctypes.byref(first)) == 0, jp._native.last_error()
    assert bad.value == 0, f"{bad.value} mismatches; first input bits {first.value:#018x}"
