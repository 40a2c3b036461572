"""GPU plain FP64 path against the reference (golden fixtures) and the oracle.

Tolerances (the reference's contract for this path):
  - pass sequence, narrow-phase visit record (every visit with orientation,
    status and per-point hit counts, in the reference's visiting order),
    collision flags and impact-zone partitions: identical;
  - positions and velocities: within 1e-12 relative (max abs difference over
    max(|reference|, 1)). Only CCD roots and zone rotations go through
    acos/cos/pow/sin, whose CUDA and glibc results may differ by an ulp.
"""
import glob
import os

import numpy as np
import pytest

from collision_gb300 import scenes
from tests.gpu_util import golden_inputs, record_sha, rel_err, scene_from_golden, zone_labels

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
RTOL = 1e-12


@pytest.fixture(scope="module")
def solver_cls():
    import torch
    assert torch.cuda.is_available()
    from collision_gb300.solver import CollisionSolver3d
    return CollisionSolver3d


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_gpu_matches_reference_golden(solver_cls, path):
    from collision_gb300.solver import ordered_visits
    g = np.load(path)
    sc = scene_from_golden(g)
    s = solver_cls(0)
    s.assembleFromScene(sc)
    s.setRecording(True)
    for step in range(len(g["x"])):
        x, v, hc = s.resolveCollision(*golden_inputs(g, sc, step))
        kinds = g["pass_kinds"][g["pass_kinds"][:, 0] == step][:, 1]
        assert np.array_equal(s.passKinds(), kinds), f"pass sequence differs at step {step}"
        rec = ordered_visits(s.visits())
        assert len(rec) == g["npairs"][step], f"visit count differs at step {step}"
        assert record_sha(rec) == str(g["pair_sha"][step]), f"visit record differs at step {step}"
        assert s.hasCollision() == bool(g["has_collision"][step])
        assert np.array_equal(hc, g["hc"][step])
        assert np.array_equal(zone_labels(s.zoneRoots()), g["zones"][step])
        assert rel_err(x, g["x"][step]) <= RTOL, f"positions step {step}: {rel_err(x, g['x'][step])}"
        assert rel_err(v, g["vel"][step]) <= RTOL, f"velocities step {step}: {rel_err(v, g['vel'][step])}"
        for i, sid in enumerate(sorted(sc.bodies)):
            com, comv = s.body(sid)
            assert rel_err(com, g["body_com"][step][i]) <= RTOL, f"body {sid} centre of mass, step {step}"
            assert rel_err(comv, g["body_comv"][step][i]) <= RTOL, f"body {sid} velocity, step {step}"
    s.close()


def _oracle_run(sc, nsteps, solver_cls, record=True, rope=True):
    from collision_gb300.solver import ordered_visits
    from oracle.ccopy import OracleSolver, REC_PAIRS
    o = OracleSolver(sc, record=REC_PAIRS if record else 0)
    s = solver_cls(0)
    s.assembleFromScene(sc)
    s.setRecording(record)
    s.setTuning(s.TUNE_ROPE_TRAVERSE, int(rope))
    x, v, hc = sc.x.copy(), sc.v.copy(), np.zeros(sc.nv, np.uint8)
    worst = [0.0, 0.0]
    for step in range(nsteps):
        xc = scenes.candidate(sc, x, v)
        r = o.step(x, xc, v, hc)
        assert r["rc"] == 0
        xg, vg, hg = s.resolveCollision(x, xc, v, hc)
        assert np.array_equal(s.passKinds(), o.passes()), f"pass sequence differs at step {step}"
        if record:
            p = o.pairs()
            assert record_sha(ordered_visits(s.visits())) == record_sha(p), f"visits differ at step {step}"
        assert np.array_equal(hg, r["has_collsn"])
        assert np.array_equal(zone_labels(s.zoneRoots()), zone_labels(r["zone_root"]))
        worst[0] = max(worst[0], rel_err(xg, r["x"]))
        worst[1] = max(worst[1], rel_err(vg, r["v"]))
        assert worst[0] <= RTOL and worst[1] <= RTOL, (step, worst)
        for sid in sorted(sc.bodies):
            for a, b in zip(s.body(sid), o.body(sid)):
                assert rel_err(a, b) <= RTOL, (step, sid, a, b)
        x, v, hc = r["x"], r["v"], r["has_collsn"]
    s.close()
    return worst


def test_gpu_vs_oracle_cloth_on_sphere_33(solver_cls):
    # the measured single-scene workload, shortened: 33x33 cloth on the icosphere
    sc = scenes.cloth_on_sphere(z=0.253)
    _oracle_run(sc, 6, solver_cls)


def test_gpu_vs_oracle_strings(solver_cls):
    sc = scenes.strings(nstr=16, nseg=128, seglen=2e-3, seed=4, box_lo=(-0.2, -0.2, -0.05),
                        box_hi=(0.2, 0.2, 0.049), z_range=(0.0502, 0.06), volume_z=(0.05, 0.08), speed=2.0)
    _oracle_run(sc, 6, solver_cls)


def test_gpu_vs_oracle_folded_self_collision(solver_cls):
    sc = scenes.folded_cloth(n=33, dt=5e-4, h=2e-3, seed=1, vscale=20.0)
    _oracle_run(sc, 6, solver_cls)


def test_gpu_vs_oracle_stack_traversal(solver_cls):
    # the traversal with a stack per thread instead of the stackless one:
    # the same visit record, pass sequence and state
    sc = scenes.folded_cloth(n=33, dt=5e-4, h=2e-3, seed=1, vscale=20.0)
    _oracle_run(sc, 6, solver_cls, rope=False)


def test_lbvh_pairs_equal_all_pairs(solver_cls):
    sc = scenes.folded_cloth(n=33, dt=5e-4, h=2e-3, seed=1, vscale=20.0)
    s = solver_cls(0)
    s.assembleFromScene(sc)
    s.resolveCollision(sc.x, scenes.candidate(sc, sc.x, sc.v), sc.v, np.zeros(sc.nv, np.uint8))
    # the warp-packet traversal, the stackless one along ropes, and the one
    # with a stack per thread
    for packet, rope in ((1, 0), (0, 1), (0, 0)):
        s.setTuning(s.TUNE_PACKET_TRAVERSE, packet)
        s.setTuning(s.TUNE_ROPE_TRAVERSE, rope)
        for moving in (False, True):
            a = s.candidatePairs(moving, brute_force=False)
            b = s.candidatePairs(moving, brute_force=True)
            ka = np.sort(np.minimum(a[:, 0], a[:, 1]).astype(np.int64) * sc.ne + np.maximum(a[:, 0], a[:, 1]))
            kb = np.sort(np.minimum(b[:, 0], b[:, 1]).astype(np.int64) * sc.ne + np.maximum(b[:, 0], b[:, 1]))
            assert len(ka) > 0 and np.array_equal(ka, kb), (packet, rope)
    s.close()


@pytest.mark.parametrize("host_tree", [0, 1])
def test_leaf_ranks_match_oracle(solver_cls, host_tree):
    # the trees built on the GPU (default) and by the host emulation
    from oracle.ccopy import OracleSolver
    sc = scenes.cloth_on_sphere(n=12, z=0.252, radius=0.25, sub=2, side=0.4, speed=3.0, seed=2)
    o = OracleSolver(sc, record=0)
    s = solver_cls(0)
    s.setTuning(s.TUNE_HOST_TREE, host_tree)
    s.assembleFromScene(sc)
    x, v, hc = sc.x.copy(), sc.v.copy(), np.zeros(sc.nv, np.uint8)
    for _ in range(3):
        xc = scenes.candidate(sc, x, v)
        r = o.step(x, xc, v, hc)
        s.resolveCollision(x, xc, v, hc)
        for which in (0, 1):
            assert np.array_equal(s.leafRanks(which), o.leaf_rank(which))
        x, v, hc = r["x"], r["v"], r["has_collsn"]
    s.close()


def test_empty_and_ragged_meshes(solver_cls):
    s = solver_cls(0)
    # no elements at all: candidates pass through untouched
    s.assembleFromMesh(5)
    x = np.random.default_rng(0).random((5, 3))
    xc = x + 1e-3
    xo, vo, ho = s.resolveCollision(x, xc, np.ones((5, 3)), np.zeros(5, np.uint8))
    assert np.array_equal(xo, xc) and np.array_equal(vo, np.ones((5, 3)))
    # one triangle plus an isolated point that no element references
    sc = scenes.cloth_on_sphere(n=2, sub=0, side=0.1)
    sc.tris = sc.tris[:1]
    sc.tri_surf = sc.tri_surf[:1]
    sc.tri_rest = sc.tri_rest[:1]
    s.assembleFromScene(sc)
    xc = scenes.candidate(sc, sc.x, sc.v)
    xo, vo, ho = s.resolveCollision(sc.x, xc, sc.v, np.zeros(sc.nv, np.uint8))
    from oracle.ccopy import OracleSolver
    r = OracleSolver(sc, record=0).step(sc.x, xc, sc.v, np.zeros(sc.nv, np.uint8))
    assert rel_err(xo, r["x"]) <= RTOL and rel_err(vo, r["v"]) <= RTOL
    s.close()


def test_bad_inputs_are_rejected(solver_cls):
    from collision_gb300._lib import CCError
    s = solver_cls(0)
    with pytest.raises(CCError):
        s.assembleFromMesh(3, tris=np.array([[0, 1, 5]]), tri_rest=np.ones((1, 3)))
    with pytest.raises(CCError):
        s.assembleFromMesh(3, tris=np.array([[0, 1, 1]]), tri_rest=np.ones((1, 3)))
    sc = scenes.cloth_on_sphere(n=4, sub=1, side=0.2)
    s.assembleFromScene(sc)
    x = sc.x.copy()
    xc = scenes.candidate(sc, x, sc.v)
    xc[3, 0] = np.nan
    with pytest.raises(CCError) as ei:
        s.resolveCollision(x, xc, sc.v, np.zeros(sc.nv, np.uint8))
    assert ei.value.status == 5  # CC_NAN_DETECTED; the reference exits the process here
    # the solver stays usable after the error
    xc = scenes.candidate(sc, x, sc.v)
    s.resolveCollision(x, xc, sc.v, np.zeros(sc.nv, np.uint8))
    s.close()


@pytest.mark.parametrize("make", [
    lambda: scenes.cloth_on_sphere(n=12, z=0.252, radius=0.25, sub=2, side=0.4, mu=0.3, speed=3.0, seed=2),
    lambda: scenes.folded_cloth(n=33, dt=5e-4, h=2e-3, seed=1, vscale=20.0),
    lambda: scenes.strings(nstr=16, nseg=128, seglen=2e-3, seed=4, box_lo=(-0.2, -0.2, -0.05),
                           box_hi=(0.2, 0.2, 0.049), z_range=(0.0502, 0.06), volume_z=(0.05, 0.08), speed=2.0),
], ids=["sphere_zones", "folded", "strings"])
def test_mixed_precision_equals_plain(solver_cls, make):
    """The FP32 filters only skip sub-tests that cannot hit: the mixed path's
    results, visit records and zones are the plain FP64 path's, bit for bit."""
    from collision_gb300.solver import ordered_visits
    sc = make()
    plain, mixed = solver_cls(0), solver_cls(0)
    for s, mode in ((plain, 0), (mixed, 1)):
        s.assembleFromScene(sc)
        s.setMode(mode)
        s.setRecording(True)
    x, v, hc = sc.x.copy(), sc.v.copy(), np.zeros(sc.nv, np.uint8)
    for step in range(8):
        xc = scenes.candidate(sc, x, v)
        a = plain.resolveCollision(x, xc, v, hc)
        b = mixed.resolveCollision(x, xc, v, hc)
        for u, w in zip(a, b):
            assert np.array_equal(u, w), f"step {step}"
        assert record_sha(ordered_visits(plain.visits())) == record_sha(ordered_visits(mixed.visits()))
        assert np.array_equal(zone_labels(plain.zoneRoots()), zone_labels(mixed.zoneRoots()))
        x, v, hc = a
    plain.close()
    mixed.close()


def test_strain_sweeps_agree(solver_cls):
    """The shared-memory window sweep and the global-memory sweep of the strain
    limiter give the same velocities (both follow the reference's order)."""
    sc = scenes.folded_cloth(n=33, dt=5e-4, h=2e-3, seed=1, vscale=20.0)
    a, b = solver_cls(0), solver_cls(0)
    for s, win in ((a, True), (b, False)):
        s.assembleFromScene(sc)
        s.setStrainWindow(win)
    x, v, hc = sc.x.copy(), sc.v.copy(), np.zeros(sc.nv, np.uint8)
    for step in range(6):
        xc = scenes.candidate(sc, x, v)
        ra = a.resolveCollision(x, xc, v, hc)
        rb = b.resolveCollision(x, xc, v, hc)
        for u, w in zip(ra, rb):
            assert np.array_equal(u, w)
        assert a.counters()["strain_averaged"] == b.counters()["strain_averaged"] > 0 or step == 0
        x, v, hc = ra
    a.close()
    b.close()


def test_wide_strain_window_agrees(solver_cls):
    """A cloth whose strain levels are wider than the sweep's block (385x385:
    up to ~290 edges a level, ~1,250 shared-memory slots) takes the window
    sweep that holds a thread's later edges of a level in registers; its
    velocities equal the global-memory sweep's."""
    sc = scenes.large(n=385)
    a, b = solver_cls(0), solver_cls(0)
    for s, win in ((a, True), (b, False)):
        s.assembleFromScene(sc)
        s.setStrainWindow(win)
    x, v, hc = sc.x.copy(), sc.v.copy(), np.zeros(sc.nv, np.uint8)
    averaged = 0
    for step in range(4):
        xc = scenes.candidate(sc, x, v)
        ra = a.resolveCollision(x, xc, v, hc)
        rb = b.resolveCollision(x, xc, v, hc)
        for u, w in zip(ra, rb):
            assert np.array_equal(u, w), step
        assert a.counters()["strain_averaged"] == b.counters()["strain_averaged"]
        averaged += a.counters()["strain_averaged"]
        x, v, hc = ra
    assert averaged > 0
    a.close()
    b.close()
