"""The correctly rounded cos/sin/acos/pow of the FP64 path (host build of
collision_gb300/csrc/cc_crmath.cuh): correctly rounded on every sample, and
equal to glibc wherever glibc is correctly rounded."""
import numpy as np
import pytest

from tests.crmath_util import evaluate, load, samples

NAMES = {0: "cos", 1: "sin", 2: "acos", 3: "pow"}


@pytest.mark.parametrize("fn", [0, 1, 2, 3], ids=[NAMES[i] for i in range(4)])
def test_correctly_rounded_against_mpmath(fn):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 200
    ref = {0: mpmath.cos, 1: mpmath.sin, 2: mpmath.acos, 3: lambda x, y: mpmath.power(x, y)}[fn]
    lib = load()
    a, b = samples(n=1500)[fn]
    ours = evaluate(lib, "cr_eval", fn, a, b)
    glibc = evaluate(lib, "libm_eval", fn, a, b)
    not_cr_ours = not_cr_glibc = 0
    for i in range(len(a)):
        args = [mpmath.mpf(a[i])] + ([mpmath.mpf(b[i])] if b is not None else [])
        r = float(ref(*args))
        not_cr_ours += ours[i] != r
        not_cr_glibc += glibc[i] != r
        # wherever glibc is correctly rounded, we agree with it
        if glibc[i] == r:
            assert ours[i] == glibc[i]
    assert not_cr_ours == 0
    assert not_cr_glibc <= 0.01 * len(a)


def test_special_values():
    lib = load()
    assert evaluate(lib, "cr_eval", 2, np.array([1.0]))[0] == 0.0
    assert evaluate(lib, "cr_eval", 2, np.array([-1.0]))[0] == np.pi
    assert np.isnan(evaluate(lib, "cr_eval", 2, np.array([1.0 + 2.0 ** -52]))[0])
    assert evaluate(lib, "cr_eval", 1, np.array([0.0]))[0] == 0.0
    assert evaluate(lib, "cr_eval", 3, np.array([0.0]), np.array([1.0 / 3.0]))[0] == 0.0
