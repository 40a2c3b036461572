"""The host emulation of the reference tree's insertion order, on the CPU.

The leaf ranks of the reference's incremental AABB trees (AABB.cpp:129-197)
orient every pair and order every sum, so the runtime rebuilds them on the
host (collision_gb300/csrc/cc_tree_order.cpp). Here that file is compiled
with g++ and its ranks are compared with the oracle's trees after one step:
the static tree from x_old boxes, and - on a step without impulses, where the
first CCD pass sees avgVel = (x_cand - x_old)/dt - the swept tree.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from collision_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = "/usr/local/cuda/include"


@pytest.fixture(scope="module")
def tree_ranks(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx or not os.path.isdir(CUDA_INC):
        pytest.skip("needs g++ and the CUDA headers")
    so = str(tmp_path_factory.mktemp("tree_order") / "libtree_order.so")
    src = os.path.join(ROOT, "collision_gb300", "csrc")
    subprocess.run([gxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off", "-I", src, "-I", CUDA_INC,
                    os.path.join(ROOT, "tests", "tree_order_shim.cpp"), os.path.join(src, "cc_tree_order.cpp"),
                    "-o", so], check=True)
    lib = C.CDLL(so)
    lib.tree_ranks.restype = C.c_double
    lib.tree_ranks.argtypes = [C.c_void_p, C.c_int, C.c_void_p]

    def ranks(boxes):
        b = np.ascontiguousarray(boxes, np.float64)
        out = np.empty(len(b), np.int32)
        lib.tree_ranks(b.ctypes.data, len(b), out.ctypes.data)
        return out
    return ranks


def _leaf_boxes(sc, x, x_end=None):
    """Leaf boxes as the reference forms them (AABB.cpp:6-36): the extent of
    the element's points at x (and at x_end for swept boxes), padded by 1e-6."""
    boxes = []
    for pts in (np.asarray(sc.tris, np.int64), np.asarray(sc.bonds, np.int64)):
        if len(pts) == 0:
            continue
        p = x[pts] if x_end is None else np.concatenate([x[pts], x_end[pts]], axis=1)
        boxes.append(np.concatenate([p.min(axis=1) - 1e-6, p.max(axis=1) + 1e-6], axis=1))
    return np.concatenate(boxes)


@pytest.mark.parametrize("make", [
    lambda: scenes.cloth_on_sphere(n=12, z=0.30, radius=0.25, sub=2, side=0.4, speed=1.0, seed=2),
    lambda: scenes.cloth_on_sphere(n=33, seed=0),
    lambda: scenes.strings(nstr=4, nseg=64, seed=4),
    lambda: scenes.folded_cloth(n=17, seed=1),
], ids=["cloth12", "cloth33", "strings", "folded17"])
def test_tree_ranks_match_oracle(tree_ranks, make):
    from oracle.ccopy import OracleSolver
    sc = make()
    x = sc.x.copy()
    xc = scenes.candidate(sc, x, sc.v)
    o = OracleSolver(sc, record=0)
    r = o.step(x, xc, sc.v.copy(), np.zeros(sc.nv, np.uint8))
    assert r["rc"] == 0
    assert np.array_equal(tree_ranks(_leaf_boxes(sc, x)), o.leaf_rank(0))
    if not r["has_collsn"].any():
        # no impulse in the step: the first CCD pass swept x_old by
        # avgVel = (x_cand - x_old)/dt
        dt = sc.params["dt"]
        x_end = x + ((xc - x) / dt) * dt
        assert np.array_equal(tree_ranks(_leaf_boxes(sc, x, x_end)), o.leaf_rank(1))
