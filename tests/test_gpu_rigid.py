"""Movable rigid bodies and the reference's decks on the GPU.

A movable body (a surface of points flagged 2) is one impact zone for the
whole step (createImpZoneForRG, dcollid3d.cpp:54-68), takes spread impulses
from rigid-rigid contacts (SpreadImpactZoneImpulse, dcollid.cpp:1101-1115),
moves rigidly after every pass (updateImpactZoneVelocityForRG,
dcollid.cpp:267-288) and reports its centre of mass and velocity at the end
(updateFinalForRG, dcollid.cpp:626-675). The golden fixtures pin a few steps
against the reference itself (test_gpu_parity.py); here longer runs are
checked against the oracle, batches against single scenes, and the mixed
precision path against the plain one.
"""
import numpy as np
import pytest

from collision_gb300 import scenes
from tests.golden import cases
from tests.gpu_util import rel_err, zone_labels
from tests.test_gpu_parity import RTOL, _oracle_run

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def solver_cls():
    from collision_gb300.solver import CollisionSolver3d
    return CollisionSolver3d


RIGID = ["rigid_bodies", "sphere12_movable", "deck_ball_plane", "deck_string_slide"]


@pytest.mark.parametrize("name", RIGID)
def test_rigid_vs_oracle(solver_cls, name):
    make, _ = cases.CASES[name]
    _oracle_run(make(), 16, solver_cls)


@pytest.mark.parametrize("name", ["deck_ball_ball", "deck_string_box", "deck_string_string"])
def test_decks_vs_oracle(solver_cls, name):
    make, _ = cases.CASES[name]
    _oracle_run(make(), 12, solver_cls)


def _run(solver_cls, mix, nsteps, mode, batch):
    """States after each step, per scene, solved as one batch or one by one."""
    out = []
    if batch:
        s = solver_cls(0)
        s.assembleBatch(mix)
        s.setMode(mode)
        off, _ = s.sceneOffsets()
        x = np.concatenate([sc.x for sc in mix])
        v = np.concatenate([sc.v for sc in mix])
        dt = np.concatenate([np.full((sc.nv, 1), sc.params["dt"]) for sc in mix])
        hc = np.zeros(len(x), np.uint8)
        for _ in range(nsteps):
            x, v, hc, _ = s.resolveCollisionBatch(x, x + dt * v, v, hc)
            out.append([dict(x=x[off[i]:off[i + 1]], v=v[off[i]:off[i + 1]], hc=hc[off[i]:off[i + 1]],
                             bodies={b: s.body(b, scene=i) for b in sorted(sc.bodies)})
                        for i, sc in enumerate(mix)])
        s.close()
        return out
    per = []
    for sc in mix:
        s = solver_cls(0)
        s.assembleFromScene(sc)
        s.setMode(mode)
        x, v, hc = sc.x.copy(), sc.v.copy(), np.zeros(sc.nv, np.uint8)
        states = []
        for _ in range(nsteps):
            x, v, hc = s.resolveCollision(x, scenes.candidate(sc, x, v), v, hc)
            states.append(dict(x=x, v=v, hc=hc, bodies={b: s.body(b) for b in sorted(sc.bodies)}))
        s.close()
        per.append(states)
    return [[per[i][k] for i in range(len(mix))] for k in range(nsteps)]


def _same(a, b, tag):
    for k, (sa, sb) in enumerate(zip(a, b)):
        for i, (p, q) in enumerate(zip(sa, sb)):
            assert np.array_equal(p["x"], q["x"]), (tag, k, i)
            assert np.array_equal(p["v"], q["v"]), (tag, k, i)
            assert np.array_equal(p["hc"], q["hc"]), (tag, k, i)
            for sid in p["bodies"]:
                for u, w in zip(p["bodies"][sid], q["bodies"][sid]):
                    assert np.array_equal(u, w), (tag, k, i, sid)


def test_rigid_batch_equals_single_and_mixed_equals_plain(solver_cls):
    mix = [cases.CASES["rigid_bodies"][0](), scenes.cloth_on_sphere(n=9, z=0.2525, radius=0.25, sub=2, side=0.3),
           cases.CASES["deck_ball_plane"][0](), cases.CASES["deck_string_slide"][0]()]
    ref = _run(solver_cls, mix, 10, 0, batch=False)
    _same(ref, _run(solver_cls, mix, 10, 0, batch=True), "plain batch")
    _same(ref, _run(solver_cls, mix, 10, 1, batch=True), "mixed batch")
    _same(ref, _run(solver_cls, mix, 10, 1, batch=False), "mixed single")
    # the bodies did collide and move
    assert any(np.any(st[0]["hc"][:42]) for st in ref)


def test_rigid_input_checks(solver_cls):
    from collision_gb300._lib import CCError as CollisionError
    base = cases.CASES["rigid_bodies"][0]()
    bad = []
    sc = base.copy()
    sc.fixed[0] = 3  # both flags
    bad.append(sc)
    sc = base.copy()
    sc.fixed[5] = 0  # a non-movable point inside a movable surface
    bad.append(sc)
    sc = base.copy()
    sc.fixed[-1] = 2  # a movable cloth point
    bad.append(sc)
    for sc in bad:
        s = solver_cls(0)
        with pytest.raises(CollisionError):
            s.assembleFromScene(sc)
        s.close()
    s = solver_cls(0)
    s.assembleFromScene(base)
    with pytest.raises(CollisionError):
        s.setBody(2, 1.0, np.zeros(3), np.zeros(3))  # surface 2 is the fixed box
    s.close()
