"""The reference trees' leaf order built on the GPU against the host
emulation of the reference's insertions (collision_gb300/csrc/cc_tree_order.cpp,
itself compared with the oracle's trees in tests/test_tree_order_cpu.py).

Both trees of every scene (the static one of the proximity pass and the
swept one of the first CCD pass) after one step: every leaf's rank and the
shared root volume bit for bit, and the step's results. The cases include
flat cloth, where most insertions descend along long chains and many
volume comparisons tie (ties go right), duplicated triangles (identical
boxes), the 64 x 512 strings, the 257x257 cloth of the large workload and a
16-scene batch.
"""
import numpy as np
import pytest

from collision_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def solver_cls():
    import torch
    assert torch.cuda.is_available()
    from collision_gb300.solver import CollisionSolver3d
    return CollisionSolver3d


def _duplicated_soup():
    # a flat cloth over a sphere with every triangle listed twice
    sc = scenes.cloth_on_sphere(n=17, z=0.27, radius=0.25, sub=1, side=0.4, speed=1.0, seed=5)
    tris = np.concatenate([sc.tris, sc.tris[::-1]])
    surf = np.concatenate([sc.tri_surf, sc.tri_surf[::-1]])
    rest = np.concatenate([sc.tri_rest, sc.tri_rest[::-1]])
    order = np.argsort(surf, kind="stable")  # surfaces stay contiguous runs
    return scenes.Scene(**{**sc.__dict__, "name": "dup_soup", "tris": np.ascontiguousarray(tris[order]),
                           "tri_surf": np.ascontiguousarray(surf[order]),
                           "tri_rest": np.ascontiguousarray(rest[order])})


CASES = {
    "cloth_on_sphere_33": lambda: [scenes.cloth_on_sphere()],
    "folded_cloth_65": lambda: [scenes.folded_cloth(n=65)],
    "strings_64x512": lambda: [scenes.strings()],
    "large_257": lambda: [scenes.large(n=257)],
    "batch_16": lambda: scenes.batched(nscenes=16, seed=3),
}


def _run(solver_cls, scs, host_tree):
    s = solver_cls(0)
    s.setTuning(s.TUNE_HOST_TREE, host_tree)
    if len(scs) == 1:
        s.assembleFromScene(scs[0])
        sc = scs[0]
        out = s.resolveCollision(sc.x, scenes.candidate(sc, sc.x, sc.v), sc.v, np.zeros(sc.nv, np.uint8))
    else:
        s.assembleBatch(scs)
        x = np.concatenate([sc.x for sc in scs])
        v = np.concatenate([sc.v for sc in scs])
        dt = np.concatenate([np.full((sc.nv, 1), sc.params["dt"]) for sc in scs])
        out = s.resolveCollisionBatch(x, x + dt * v, v, np.zeros(len(x), np.uint8))
    r = (s.leafRanks(0), s.leafRanks(1), [s.treeVolume(i) for i in range(len(scs))], out,
         s.counters()["tree_builds"])
    s.close()
    return r


@pytest.mark.parametrize("case", sorted(CASES))
def test_gpu_tree_order_equals_host_emulation(solver_cls, case):
    scs = CASES[case]()
    g = _run(solver_cls, scs, 0)
    h = _run(solver_cls, scs, 1)
    assert g[0] is not None and g[1] is not None
    assert np.array_equal(g[0], h[0]), f"{case}: static tree ranks"
    assert np.array_equal(g[1], h[1]), f"{case}: swept tree ranks"
    assert g[2] == h[2], f"{case}: root volumes"
    for a, b in zip(g[3], h[3]):
        assert np.array_equal(a, b), f"{case}: step results"
    assert g[4] == h[4] >= len(scs)


def test_gpu_tree_order_duplicates(solver_cls):
    sc = _duplicated_soup()
    g = _run(solver_cls, [sc], 0)
    h = _run(solver_cls, [sc], 1)
    assert np.array_equal(g[0], h[0]) and np.array_equal(g[1], h[1]) and g[2] == h[2]
