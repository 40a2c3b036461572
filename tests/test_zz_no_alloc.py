"""cc_candidate_pairs_static: the candidate-pair search for callers that
cannot allocate device memory (their memory belongs to another allocator, or
they must not stall on cudaMalloc). It works out of a fixed scratch area in
the library, so these checks run it twice in a row on different meshes and
compare each result with the pairs the allocating solver finds for the same
boxes; the pair sets are integers and must be identical.

This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from collision_gb300 import scenes

pytestmark = pytest.mark.gpu


def static_boxes(sc, x):
    """The solver's proximity boxes: per element, min/max of its points'
    x_old padded by 1e-6 (AABB.cpp:10-11)."""
    boxes = []
    if sc.nt:
        p = x[sc.tris]
        boxes.append(np.concatenate([p.min(axis=1) - 1e-6, p.max(axis=1) + 1e-6], axis=1))
    if sc.nb:
        p = x[sc.bonds]
        boxes.append(np.concatenate([p.min(axis=1) - 1e-6, p.max(axis=1) + 1e-6], axis=1))
    return np.ascontiguousarray(np.concatenate(boxes), dtype=np.float64)


def pair_keys(pairs, ne):
    a = np.minimum(pairs[:, 0], pairs[:, 1]).astype(np.int64)
    b = np.maximum(pairs[:, 0], pairs[:, 1]).astype(np.int64)
    return np.sort(a * ne + b)


def test_static_pairs_match_allocating_path_twice():
    import torch
    from collision_gb300 import _lib
    from collision_gb300.solver import CollisionSolver3d
    lib = _lib.load()
    cases = [scenes.folded_cloth(n=33, dt=5e-4, h=2e-3, seed=1, vscale=20.0),
             scenes.strings(nstr=16, nseg=64, seglen=2e-3, seed=4, box_lo=(-0.2, -0.2, -0.05),
                            box_hi=(0.2, 0.2, 0.049), z_range=(0.0502, 0.06), volume_z=(0.05, 0.08))]
    for sc in cases:
        s = CollisionSolver3d(0)
        s.assembleFromScene(sc)
        s.resolveCollision(sc.x, scenes.candidate(sc, sc.x, sc.v), sc.v, np.zeros(sc.nv, np.uint8))
        expected = s.candidatePairs(moving=False)  # existing, allocating entry point
        s.close()
        boxes = torch.tensor(static_boxes(sc, sc.x), device="cuda:0")
        cap = len(expected) + 1024
        out = torch.full((cap, 2), -1, dtype=torch.int32, device="cuda:0")
        torch.cuda.synchronize()
        n = C.c_int(-1)
        st = lib.cc_candidate_pairs_static(0, boxes.data_ptr(), sc.ne, out.data_ptr(), cap, C.byref(n), None)
        assert st == 0
        assert n.value == len(expected) > 0
        got = out[: n.value].cpu().numpy()
        assert np.array_equal(pair_keys(got, sc.ne), pair_keys(expected, sc.ne))


def test_static_pairs_reject_oversize():
    from collision_gb300 import _lib
    lib = _lib.load()
    n = C.c_int(-1)
    st = lib.cc_candidate_pairs_static(0, None, 65537, None, 0, C.byref(n), None)
    assert st == 1  # CC_BAD_INPUT
    buf = C.create_string_buffer(256)
    lib.cc_static_last_error(buf, 256)
    assert b"65536" in buf.value
