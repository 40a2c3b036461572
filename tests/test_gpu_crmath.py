"""The GPU evaluates the correctly rounded math bit-identically to the host
build of the same source."""
import ctypes as C

import numpy as np
import pytest

from tests.crmath_util import evaluate, load, samples

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fn", [0, 1, 2, 3])
def test_device_equals_host(fn):
    from collision_gb300 import _lib
    lib = _lib.load()
    host = load()
    a, b = samples(seed=11, n=4000)[fn]
    b_arr = np.ascontiguousarray(a if b is None else b, dtype=np.float64)
    a = np.ascontiguousarray(a, dtype=np.float64)
    out = np.zeros_like(a)
    n = lib.cc_selftest_math(0, fn, a.ctypes.data, b_arr.ctypes.data, out.ctypes.data, len(a))
    assert n == len(a)
    ref = evaluate(host, "cr_eval", fn, a, b)
    assert np.array_equal(out, ref, equal_nan=True)
