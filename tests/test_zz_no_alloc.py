"""cc_candidate_pairs_static: the candidate-pair search for callers that
cannot allocate device memory (their memory belongs to another allocator, or
they must not stall on cudaMalloc). It works out of a fixed scratch area in
the library, so these checks run it twice in a row on different meshes and
compare each result with the pairs the allocating solver finds for the same
boxes; the pair sets are integers and must be identical. It also runs at its
documented limit of 65,536 boxes, with a cap below the pair count, and on
boxes it must reject.

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


def _call(lib, boxes, n, out, cap):
    import torch
    torch.cuda.synchronize()
    cnt = C.c_int(-1)
    st = lib.cc_candidate_pairs_static(0, boxes.data_ptr(), n, out.data_ptr(), cap, C.byref(cnt), None)
    return st, cnt.value


def test_static_pairs_at_the_limit():
    """65,536 boxes, the documented maximum, where the scratch layout is
    tightest: a 256 x 256 grid of unit cells, each box overlapping exactly
    its eight neighbours, in a shuffled order; the pair set is known."""
    import torch
    from collision_gb300 import _lib
    lib = _lib.load()
    m = 256
    i, j = np.meshgrid(np.arange(m), np.arange(m), indexing="ij")
    i, j = i.ravel(), j.ravel()
    perm = np.random.default_rng(5).permutation(m * m)
    ci, cj = i[perm], j[perm]  # cell of box k
    z = np.random.default_rng(6).uniform(0.0, 0.05, m * m)
    lo = np.stack([ci - 0.5 - 1e-3, cj - 0.5 - 1e-3, z - 0.1], axis=1)
    hi = np.stack([ci + 0.5 + 1e-3, cj + 0.5 + 1e-3, z + 0.1], axis=1)
    boxes = torch.tensor(np.ascontiguousarray(np.concatenate([lo, hi], axis=1)), device="cuda:0")
    where = np.empty(m * m, np.int64)
    where[ci * m + cj] = np.arange(m * m)
    exp = []
    for di, dj in ((1, 0), (0, 1), (1, 1), (1, -1)):
        ok = (i + di < m) & (j + dj >= 0) & (j + dj < m)
        a = where[i[ok] * m + j[ok]]
        b = where[(i[ok] + di) * m + j[ok] + dj]
        exp.append(np.stack([a, b], axis=1))
    exp = pair_keys(np.concatenate(exp), m * m)
    cap = len(exp) + 16
    out = torch.full((cap, 2), -1, dtype=torch.int32, device="cuda:0")
    for _ in range(2):
        st, n = _call(lib, boxes, m * m, out, cap)
        assert st == 0 and n == len(exp)
        assert np.array_equal(pair_keys(out[:n].cpu().numpy(), m * m), exp)


def test_static_pairs_overflow_and_bad_boxes():
    """A cap below the pair count writes cap pairs of the set and reports the
    full count; a NaN or inverted box is rejected; a good call after either
    gives the full set again."""
    import torch
    from collision_gb300 import _lib
    from collision_gb300.solver import CollisionSolver3d
    lib = _lib.load()
    sc = scenes.folded_cloth(n=33, dt=5e-4, h=2e-3, seed=1, vscale=20.0)
    s = CollisionSolver3d(0)
    s.assembleFromScene(sc)
    s.resolveCollision(sc.x, scenes.candidate(sc, sc.x, sc.v), sc.v, np.zeros(sc.nv, np.uint8))
    expected = pair_keys(s.candidatePairs(moving=False), sc.ne)
    s.close()
    good = static_boxes(sc, sc.x)
    boxes = torch.tensor(good, device="cuda:0")
    cap = 100
    out = torch.full((len(expected) + 64, 2), -1, dtype=torch.int32, device="cuda:0")
    st, n = _call(lib, boxes, sc.ne, out, cap)
    assert st == 2 and n == len(expected) > cap  # CC_PAIR_OVERFLOW with the full count
    got = pair_keys(out[:cap].cpu().numpy(), sc.ne)
    assert len(np.unique(got)) == cap and np.isin(got, expected).all()
    assert (out[cap:].cpu().numpy() == -1).all()  # nothing written past cap
    for bad in ("nan", "inverted"):
        b = good.copy()
        if bad == "nan":
            b[7, 1] = np.nan
        else:
            b[11, 2], b[11, 5] = b[11, 5] + 1e-3, b[11, 2]
        st, n = _call(lib, torch.tensor(b, device="cuda:0"), sc.ne, out, len(out))
        assert st == 1 and n == 0, bad  # CC_BAD_INPUT
        buf = C.create_string_buffer(256)
        lib.cc_static_last_error(buf, 256)
        assert b"NaN" in buf.value
    st, n = _call(lib, boxes, sc.ne, out, len(out))
    assert st == 0 and np.array_equal(pair_keys(out[:n].cpu().numpy(), sc.ne), expected)


def test_static_pairs_reject_oversize():
    from collision_gb300 import _lib
    lib = _lib.load()
    n = C.c_int(-1)
    st = lib.cc_candidate_pairs_static(0, None, 65537, None, 0, C.byref(n), None)
    assert st == 1  # CC_BAD_INPUT
    buf = C.create_string_buffer(256)
    lib.cc_static_last_error(buf, 256)
    assert b"65536" in buf.value
