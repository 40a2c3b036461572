"""Host build of the correctly rounded math (tests/crmath_host.cpp)."""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "crmath_host.cpp")
HDR = os.path.join(os.path.dirname(HERE), "collision_gb300", "csrc", "cc_crmath.cuh")
OUT_DIR = os.path.join(os.path.dirname(HERE), "oracle", "_build")
LIB = os.path.join(OUT_DIR, "libcrmath_host.so")
_dp = C.POINTER(C.c_double)


def load():
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(SRC), os.path.getmtime(HDR)):
        os.makedirs(OUT_DIR, exist_ok=True)
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", tmp, SRC])
        os.replace(tmp, LIB)
    return C.CDLL(LIB)


def evaluate(lib, which, fn, a, b=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(a if b is None else b, dtype=np.float64)
    out = np.zeros_like(a)
    getattr(lib, which)(fn, a.ctypes.data_as(_dp), b.ctypes.data_as(_dp), out.ctypes.data_as(_dp), len(a))
    return out


def samples(seed=7, n=3000):
    """Arguments in the ranges the CCD root finder and the zone rotation use."""
    rng = np.random.default_rng(seed)
    th = rng.uniform(0, np.pi, n)
    return {
        0: (np.concatenate([th / 3, (th + 2 * np.pi) / 3, (th - 2 * np.pi) / 3, rng.uniform(-1e-3, 1e-3, n)]), None),
        1: (np.concatenate([rng.uniform(0, 1e-2, n), 10 ** rng.uniform(-12, 0, n)]), None),
        2: (np.concatenate([rng.uniform(-1, 1, n), 1 - 10 ** rng.uniform(-16, -0.3, n),
                            -1 + 10 ** rng.uniform(-16, -0.3, n), np.array([1.0, -1.0, 0.0, 0.5, -0.5])]), None),
        3: (10 ** rng.uniform(-30, 30, n), np.full(n, 1.0 / 3.0)),
    }
