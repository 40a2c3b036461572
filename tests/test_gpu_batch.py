"""Batched path: several independent scenes resolved together.

A batch must give every scene exactly what a solver holding that scene alone
gives it (same bits: the per-scene arithmetic, trees, pass sequence and
summation order do not depend on the other scenes), and so, through the
single-scene parity tests, what the reference gives it. Checked here on a
mix of sizes, element kinds and parameters, with scenes that finish after
one CCD pass next to scenes that need impact zones, plus an empty scene.
"""
import numpy as np
import pytest

from collision_gb300 import scenes
from tests.gpu_util import record_sha, rel_err, zone_labels

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _points_only(n=7, seed=3):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, size=(n, 3))
    return scenes.Scene("points_only", x, rng.uniform(-1, 1, size=(n, 3)), np.zeros(n, np.uint8),
                        np.zeros((0, 3), np.int32), np.zeros(0, np.int32), np.zeros((0, 3)),
                        np.zeros((0, 2), np.int32), np.zeros(0, np.int32), np.zeros(0),
                        np.array([-10, -10, -10, 10, 10, 10], np.float64), dict(scenes.DEFAULTS))


def _mix():
    out = [
        scenes.cloth_on_obstacle(10, "sphere", 0.2, 1.5, seed=1),
        scenes.folded_cloth(n=17, seed=1),
        scenes.cloth_on_obstacle(14, "box", 0.2, 2.5, seed=2),
        _points_only(),
        scenes.strings(nstr=4, nseg=32, seed=4),
        scenes.cloth_on_sphere(n=12, speed=3.0, seed=5),
    ]
    # a tight domain box on one scene exercises the per-scene clamp
    out[2].domain = np.array([-0.6, -0.6, -0.01, 0.6, 0.6, 1.0])
    return out


@pytest.fixture(scope="module")
def solver_cls():
    import torch
    assert torch.cuda.is_available()
    from collision_gb300.solver import CollisionSolver3d
    return CollisionSolver3d


def _split(a, off, i):
    return a[off[i]:off[i + 1]]


def _run_batch(solver_cls, mix, nsteps, mode=0, window=True, record=False, split=True, graph=True, combined=True,
               warp=False, packet=False, roles=True, overlap=False, rope=True, subset_refit=True, device_loop=True,
               refill=8, zone_cap=None, pair_capacity=None, small_sort=True, pruned_warp=True, robust_roots=True,
               zone_cta_min=None, replay_cta_min=None, refit_up=True, zone_few=None, sub_merge=True):
    b = solver_cls(0)
    b.assembleBatch(mix)
    b.setMode(mode)
    b.setTuning(solver_cls.TUNE_REFIT_UP, int(refit_up))
    b.setTuning(solver_cls.TUNE_SUBTEST_MERGE, int(sub_merge))
    if zone_few is not None:
        b.setTuning(solver_cls.TUNE_ZONE_FEW, zone_few)
    if zone_cta_min is not None:
        b.setTuning(solver_cls.TUNE_ZONE_CTA_MIN, zone_cta_min)
    if replay_cta_min is not None:
        b.setTuning(solver_cls.TUNE_REPLAY_CTA_MIN, replay_cta_min)
    b.setTuning(solver_cls.TUNE_ROBUST_ROOTS, int(robust_roots))
    b.setTuning(solver_cls.TUNE_SMALL_SORT, int(small_sort))
    b.setTuning(solver_cls.TUNE_PRUNED_WARP, int(pruned_warp))
    if pair_capacity is not None:
        b.setTuning(solver_cls.TUNE_PAIR_CAPACITY, pair_capacity)
    b.setTuning(solver_cls.TUNE_DEVICE_LOOP, int(device_loop))
    b.setTuning(solver_cls.TUNE_TRAVERSE_REFILL, int(refill))
    if zone_cap is not None:
        b.setZoneCap(zone_cap)
    b.setStrainWindow(window)
    b.setTuning(solver_cls.TUNE_SPLIT_NARROW, int(split))
    b.setTuning(solver_cls.TUNE_TAIL_GRAPH, int(graph))
    b.setTuning(solver_cls.TUNE_COMBINED_BROAD, int(combined))
    b.setTuning(solver_cls.TUNE_STRAIN_WARP, int(warp))
    b.setTuning(solver_cls.TUNE_PACKET_TRAVERSE, int(packet))
    b.setTuning(solver_cls.TUNE_ROPE_TRAVERSE, int(rope))
    b.setTuning(solver_cls.TUNE_SUBSET_REFIT, int(subset_refit))
    b.setTuning(solver_cls.TUNE_STRAIN_ROLES, int(roles))
    b.setTuning(solver_cls.TUNE_TAIL_OVERLAP, int(overlap))
    b.setRecording(record)
    pv, pe = b.sceneOffsets()
    x = np.concatenate([s.x for s in mix])
    v = np.concatenate([s.v for s in mix])
    hc = np.zeros(len(x), np.uint8)
    dt = np.concatenate([np.full(s.nv, s.params["dt"]) for s in mix])[:, None]
    steps = []
    for _ in range(nsteps):
        xc = x + dt * v
        xo, vo, ho, hcol = b.resolveCollisionBatch(x, xc, v, hc)
        info = dict(x_in=x, xc=xc, v_in=v, hc_in=hc, x=xo, v=vo, hc=ho, hcol=hcol,
                    kinds=[b.scenePassKinds(i) for i in range(len(mix))],
                    zones=b.zoneRoots(), visits=b.visits() if record else None, counters=b.counters(),
                    status=b.sceneStatus())
        steps.append(info)
        x, v, hc = xo, vo, ho
    b.close()
    return steps, pv, pe


def test_batch_equals_single_scenes(solver_cls):
    from collision_gb300.solver import ordered_visits
    mix = _mix()
    steps, pv, pe = _run_batch(solver_cls, mix, 12, record=True)
    for i, sc in enumerate(mix):
        s = solver_cls(0)
        s.assembleFromScene(sc)
        s.setRecording(True)
        for k, st in enumerate(steps):
            xs, vs, hs = s.resolveCollision(_split(st["x_in"], pv, i), _split(st["xc"], pv, i),
                                            _split(st["v_in"], pv, i), _split(st["hc_in"], pv, i))
            tag = f"scene {i} ({sc.name}) step {k}"
            assert np.array_equal(xs, _split(st["x"], pv, i)), tag
            assert np.array_equal(vs, _split(st["v"], pv, i)), tag
            assert np.array_equal(hs, _split(st["hc"], pv, i)), tag
            assert s.hasCollision() == bool(st["hcol"][i]), tag
            assert np.array_equal(s.passKinds(), st["kinds"][i]), tag
            assert np.array_equal(zone_labels(_split(st["zones"], pv, i) - pv[i]), zone_labels(s.zoneRoots())), tag
            bv = st["visits"]
            mine = bv[(bv[:, 2] >= pe[i]) & (bv[:, 2] < pe[i + 1])].copy()
            mine[:, 2:4] -= pe[i]
            assert record_sha(ordered_visits(mine)) == record_sha(ordered_visits(s.visits())), tag
        s.close()


def _first_elements(k, seed):
    # a cloth-on-sphere scene cut to its first k triangles (the other points
    # stay, referenced by no element)
    sc = scenes.cloth_on_sphere(n=2, sub=0, side=0.1, speed=2.0, seed=seed)
    sc.tris, sc.tri_surf, sc.tri_rest = sc.tris[:k], sc.tri_surf[:k], sc.tri_rest[:k]
    return sc


def test_batch_with_one_and_two_element_scenes(solver_cls):
    # scenes of one and two elements between larger ones and an empty one:
    # ropes that end at every scene boundary, and passes over some scenes
    # that refit the hierarchy around them
    mix = [_first_elements(1, 1), scenes.cloth_on_obstacle(10, "sphere", 0.2, 1.5, seed=1), _first_elements(2, 2),
           _points_only(), scenes.folded_cloth(n=17, seed=1), _first_elements(1, 3), _first_elements(2, 4)]
    singles = []
    for i, sc in enumerate(mix):
        s = solver_cls(0)
        s.assembleFromScene(sc)
        s.setMode(1)
        singles.append(s)
    ref = None
    for rope, subset_refit in ((True, True), (False, True), (True, False), (False, False)):
        steps, pv, pe = _run_batch(solver_cls, mix, 6, mode=1, rope=rope, subset_refit=subset_refit)
        if ref is None:
            ref = steps
            for i, s in enumerate(singles):
                for k, st in enumerate(steps):
                    xs, vs, hs = s.resolveCollision(_split(st["x_in"], pv, i), _split(st["xc"], pv, i),
                                                    _split(st["v_in"], pv, i), _split(st["hc_in"], pv, i))
                    tag = f"scene {i} ({mix[i].name}, {mix[i].ne} elements) step {k}"
                    assert np.array_equal(xs, _split(st["x"], pv, i)), tag
                    assert np.array_equal(vs, _split(st["v"], pv, i)), tag
                    assert np.array_equal(hs, _split(st["hc"], pv, i)), tag
                    assert np.array_equal(s.passKinds(), st["kinds"][i]), tag
        else:
            _compare(ref, steps, ("rope", rope, "subset refit", subset_refit))
    for s in singles:
        s.close()


def test_batch_matches_oracle(solver_cls):
    from oracle.ccopy import OracleSolver
    mix = _mix()
    steps, pv, pe = _run_batch(solver_cls, mix, 6)
    for i, sc in enumerate(mix):
        if sc.ne == 0:
            for st in steps:  # nothing to collide: candidates pass through
                assert np.array_equal(_split(st["x"], pv, i), _split(st["xc"], pv, i))
                assert np.array_equal(_split(st["v"], pv, i), _split(st["v_in"], pv, i))
            continue
        o = OracleSolver(sc)
        for k, st in enumerate(steps):
            r = o.step(_split(st["x_in"], pv, i), _split(st["xc"], pv, i), _split(st["v_in"], pv, i),
                       _split(st["hc_in"], pv, i))
            assert r["rc"] == 0
            tag = f"scene {i} ({sc.name}) step {k}"
            assert np.array_equal(o.passes(), st["kinds"][i]), tag
            assert np.array_equal(_split(st["hc"], pv, i), r["has_collsn"]), tag
            assert rel_err(_split(st["x"], pv, i), r["x"]) <= RTOL, tag
            assert rel_err(_split(st["v"], pv, i), r["v"]) <= RTOL, tag


def test_batch_mixed_and_global_strain_equal_plain(solver_cls):
    mix = _mix()
    ref, _, _ = _run_batch(solver_cls, mix, 8)
    for mode, window, split, graph, comb in ((1, True, True, True, True), (1, True, False, True, True),
                                             (0, False, True, True, True), (1, False, True, True, True),
                                             (0, True, True, False, True), (1, True, True, False, True),
                                             (0, True, True, True, False), (1, True, True, True, False)):
        got, _, _ = _run_batch(solver_cls, mix, 8, mode=mode, window=window, split=split, graph=graph,
                               combined=comb)
        _compare(ref, got, (mode, window, split, graph, comb))
    # the one-warp staged sweep instead of the CTA-per-scene one, and the
    # warp-packet traversal or the one with a stack per thread instead of the
    # stackless one
    for mode in (0, 1):
        got, _, _ = _run_batch(solver_cls, mix, 8, mode=mode, warp=True)
        _compare(ref, got, ("warp sweep", mode))
        got, _, _ = _run_batch(solver_cls, mix, 8, mode=mode, packet=True, rope=False)
        _compare(ref, got, ("packet traversal", mode))
        got, _, _ = _run_batch(solver_cls, mix, 8, mode=mode, rope=False)
        _compare(ref, got, ("traversal with a stack per thread", mode))
        got, _, _ = _run_batch(solver_cls, mix, 8, mode=mode, rope=False, combined=False)
        _compare(ref, got, ("stack per thread, separate proximity and CCD broad phases", mode))
        got, _, _ = _run_batch(solver_cls, mix, 8, mode=mode, subset_refit=False)
        _compare(ref, got, ("a hierarchy of their own for passes over some scenes", mode))
        got, _, _ = _run_batch(solver_cls, mix, 8, mode=mode, subset_refit=True, rope=False)
        _compare(ref, got, ("stack per thread over some scenes' leaves", mode))
        got, _, _ = _run_batch(solver_cls, mix, 8, mode=mode, roles=False)
        _compare(ref, got, ("strain sweep without separate roles", mode))
        got, _, _ = _run_batch(solver_cls, mix, 8, mode=mode, overlap=True)
        _compare(ref, got, ("ends of steps beside the other scenes' passes", mode))
        got, _, _ = _run_batch(solver_cls, mix, 8, mode=mode, overlap=True, graph=False)
        _compare(ref, got, ("overlapped ends of steps launched kernel by kernel", mode))


def _compare(ref, got, tag):
    for k, (a, b) in enumerate(zip(ref, got)):
        assert np.array_equal(a["x"], b["x"]), (tag, k)
        assert np.array_equal(a["v"], b["v"]), (tag, k)
        assert np.array_equal(a["hc"], b["hc"]), (tag, k)
        assert np.array_equal(a["hcol"], b["hcol"]), (tag, k)


def test_batch_per_scene_params(solver_cls):
    """Changing one scene's parameters changes that scene only."""
    mix = [scenes.cloth_on_obstacle(12, "sphere", 0.2, 2.0, seed=7) for _ in range(3)]
    b = solver_cls(0)
    b.assembleBatch(mix)
    # the sheets start 0.05 above the sphere at 2 m/s: within 2e-2 (the
    # thicker scene's repulsion reach) after about 15 steps
    thick = dict(mix[1].params, thickness=2e-2)
    b.setSceneParams(1, thick)
    pv, _ = b.sceneOffsets()
    x = np.concatenate([s.x for s in mix])
    v = np.concatenate([s.v for s in mix])
    hc = np.zeros(len(x), np.uint8)
    xc = x + 1e-3 * v
    for _ in range(30):
        xo, vo, ho, _ = b.resolveCollisionBatch(x, xc, v, hc)
        x, v, hc = xo, vo, ho
        xc = x + 1e-3 * v
    assert np.array_equal(_split(x, pv, 0), _split(x, pv, 2))
    assert not np.array_equal(_split(x, pv, 0), _split(x, pv, 1))
    s = solver_cls(0)
    sc = mix[1].copy()
    sc.params = thick
    s.assembleFromScene(sc)
    xs, vs, hs = sc.x, sc.v, np.zeros(sc.nv, np.uint8)
    for _ in range(30):
        xs, vs, hs = s.resolveCollision(xs, xs + 1e-3 * vs, vs, hs)
    assert np.array_equal(xs, _split(x, pv, 1))
    b.close()
    s.close()


def test_batch_device_entry(solver_cls):
    import torch
    mix = _mix()[:3]
    steps, pv, _ = _run_batch(solver_cls, mix, 3)
    b = solver_cls(0)
    b.assembleBatch(mix)
    dev = torch.device("cuda:0")
    for st in steps:
        xo = torch.from_numpy(st["x_in"]).to(dev)
        xc = torch.from_numpy(st["xc"]).to(dev)
        v = torch.from_numpy(st["v_in"]).to(dev)
        hc = torch.from_numpy(st["hc_in"]).to(dev)
        out = torch.empty_like(xo)
        hcol = b.resolveCollisionBatchDevice(xo, xc, v, hc, out)
        assert np.array_equal(out.cpu().numpy(), st["x"])
        assert np.array_equal(v.cpu().numpy(), st["v"])
        assert np.array_equal(hcol, st["hcol"])
    b.close()


def test_ccd_recheck_after_resolved_steps(solver_cls):
    """The exact CCD re-check finds nothing after a resolved step and finds
    the collisions of the unresolved candidate positions."""
    import torch
    mix = [scenes.cloth_on_obstacle(12, "sphere", 0.2, 3.0, seed=11), scenes.folded_cloth(n=17, seed=2),
           scenes.strings(nstr=4, nseg=32, seed=4)]
    b = solver_cls(0)
    b.assembleBatch(mix)
    dev = torch.device("cuda:0")
    x = torch.tensor(np.concatenate([s.x for s in mix]), device=dev)
    v = torch.tensor(np.concatenate([s.v for s in mix]), device=dev)
    dt = torch.tensor(np.concatenate([np.full((s.nv, 1), s.params["dt"]) for s in mix]), device=dev)
    hc = torch.zeros(len(x), dtype=torch.uint8, device=dev)
    unresolved = 0
    for step in range(25):
        xc = x + dt * v
        xo = torch.empty_like(x)
        b.resolveCollisionBatchDevice(x, xc, v, hc, xo)
        hits, per = b.checkCCD(x, xo)
        assert hits == 0 and not per.any(), (step, hits, per)
        h2, _ = b.checkCCD(x, xc)
        unresolved += h2
        x = xo
    assert unresolved > 0
    b.close()


def test_zone_cap_stops_one_scene_only(solver_cls):
    """Scene 186 of the 256-scene workload placed for free fall (an 80x80
    cloth 0.10 above a box) reaches an impact-zone loop that the reference
    never leaves (the oracle runs into its cap there too). In a batch, that scene stops at the cap and the
    others finish exactly as they do alone; disabled afterwards, its points
    pass through."""
    stuck = scenes.batched(nscenes=256, seed=0, approach_steps=None)[186]
    other = scenes.cloth_on_obstacle(20, "sphere", 0.2, 2.0, seed=3)
    mix = [stuck, other]
    b = solver_cls(0)
    b.assembleBatch(mix)
    b.setMode(1)
    b.setZoneCap(40)
    s = solver_cls(0)
    s.assembleFromScene(other)
    pv, _ = b.sceneOffsets()
    x = np.concatenate([q.x for q in mix])
    v = np.concatenate([q.v for q in mix])
    hc = np.zeros(len(x), np.uint8)
    xs, vs, hs = other.x, other.v, np.zeros(other.nv, np.uint8)
    capped_at = None
    for step in range(70):
        xc = x + 1e-3 * v
        xo, vo, ho, _ = b.resolveCollisionBatch(x, xc, v, hc)
        status = b.sceneStatus()
        xs, vs, hs = s.resolveCollision(xs, xs + 1e-3 * vs, vs, hs)
        assert status[1] == 0
        assert np.array_equal(_split(xo, pv, 1), xs) and np.array_equal(_split(vo, pv, 1), vs), step
        if status[0] != 0:
            assert status[0] == solver_cls.ITER_CAP
            capped_at = step
            b.setSceneEnabled(0, False)
            x, v, hc = xo, vo, ho
            xc = x + 1e-3 * v
            xo, vo, ho, _ = b.resolveCollisionBatch(x, xc, v, hc)
            assert np.array_equal(_split(xo, pv, 0), _split(xc, pv, 0))
            assert np.array_equal(_split(vo, pv, 0), _split(v, pv, 0))
            break
        x, v, hc = xo, vo, ho
    assert capped_at is not None
    b.close()
    s.close()


@pytest.mark.parametrize("mode", [1, 0])
def test_autotune_keeps_results(solver_cls, mode):
    """The autotuner changes launch shapes and buffer sizes only: a solver
    tuned after its second step produces the same bits as one that is not
    (in both arithmetic modes)."""
    mix = _mix()
    ref, pv, _ = _run_batch(solver_cls, mix, 6, mode=mode)
    b = solver_cls(0)
    b.assembleBatch(mix)
    b.setMode(mode)
    x = np.concatenate([s.x for s in mix])
    v = np.concatenate([s.v for s in mix])
    hc = np.zeros(len(x), np.uint8)
    dt = np.concatenate([np.full(s.nv, s.params["dt"]) for s in mix])[:, None]
    for k in range(6):
        xo, vo, ho, hcol = b.resolveCollisionBatch(x, x + dt * v, v, hc)
        assert np.array_equal(xo, ref[k]["x"]) and np.array_equal(vo, ref[k]["v"]), k
        if k == 1:
            got = b.autotune()
            assert got["traverse_block"] in (64, 128, 256, 512) and got["pass_ms"] > 0
        x, v, hc = xo, vo, ho
    b.close()


def test_vtk_dumps(solver_cls, tmp_path):
    """Every pass writes a .vtp per scene: element points numbered by first
    appearance, positions x_old + dt*avgVel before the pass's impulses (the
    first pass's are the candidates), red elements exactly where a point
    received an impulse."""
    import xml.etree.ElementTree as ET
    sc = scenes.cloth_on_sphere(n=12, z=0.252, radius=0.25, sub=2, side=0.4, mu=0.3, speed=3.0, seed=2)
    s = solver_cls(0)
    s.assembleFromScene(sc)
    s.setVtkDump(tmp_path)
    x, v, hc = sc.x, sc.v, np.zeros(sc.nv, np.uint8)
    nfiles = 0
    for step in range(3):
        xc = x + sc.params["dt"] * v
        x1, v1, hc1 = s.resolveCollision(x, xc, v, hc)
        npass = len(s.passKinds())
        files = sorted(tmp_path.glob("surf-*.vtp"))
        assert len(files) == nfiles + npass
        first = ET.parse(files[nfiles]).getroot()
        nfiles = len(files)
        piece = first.find("PolyData/Piece")
        assert int(piece.get("NumberOfPolys")) == sc.ne
        conn = np.array(piece.find("Polys/DataArray[@Name='connectivity']").text.split(), dtype=int)
        order, seen = [], set()
        for t in sc.tris:
            for p in t:
                if p not in seen:
                    seen.add(p)
                    order.append(p)
        assert int(piece.get("NumberOfPoints")) == len(order)
        assert np.array_equal(np.array(order)[conn.reshape(-1, 3)], sc.tris)
        pts = np.array(piece.find("Points/DataArray").text.split(), dtype=float).reshape(-1, 3)
        assert np.allclose(pts, xc[order], rtol=0, atol=1e-6 * max(1.0, np.abs(xc).max()))
        imp = np.array(piece.find("PointData/DataArray").text.split(), dtype=float).reshape(-1, 3)
        col = np.array(piece.find("CellData/DataArray").text.split(), dtype=int).reshape(-1, 3)
        hit_pt = np.zeros(sc.nv, bool)
        hit_pt[np.array(order)[np.abs(imp).sum(1) > 0]] = True
        red = col[:, 0] == 255
        assert np.array_equal(red, hit_pt[sc.tris].any(1))
        x, v, hc = x1, v1, hc1
    s.setVtkDump(None)
    s.close()


def _contact_sample(k=6, seed=0):
    # scenes of the batched workload (each cloth within four steps of its
    # obstacle), the k median sizes of evenly spaced size groups, cut to at
    # most 40 vertices per side so the test stays short
    out = []
    for sc in scenes.batched(nscenes=48, seed=seed)[::8][:k]:
        n = int(round(np.sqrt(sc.nv - (642 if "sphere" in sc.name else 8))))
        m = min(n, 40)
        obst = "sphere" if "sphere" in sc.name else "box"
        r = 0.25 if obst == "sphere" else 0.2
        speed = -float(sc.v[0, 2])
        out.append(scenes.cloth_on_obstacle(m, obst, r, speed, seed=seed + len(out), gap=2.5e-3 * speed))
    return out


@pytest.mark.parametrize("mode", [0, 1], ids=["plain", "mixed"])
def test_device_loop_equals_host_loop(solver_cls, mode):
    """Every detection pass after the proximity pass in one CUDA graph, with
    each scene's pass sequence and the impact-zone union-find on the device,
    and later passes testing only the pairs with a point the previous pass
    touched, gives every scene the same bits, pass sequence, zones, hits and
    contacts as the host-driven loop, which tests every pair - on the mix
    above and on contact-heavy cloth scenes with impact-zone passes, a capped
    zone loop included."""
    # the last case starts with a pair buffer far too small, so that passes
    # stop after their narrow phase has run, grow the buffer and run again,
    # and sorts its union records with the general sort (behind the graph's
    # conditional node) instead of the one-CTA sort
    for mix, cap, pc, small in ((_mix(), None, None, True), (_contact_sample(), 3, None, True),
                                (_contact_sample(), 3, 4096, False)):
        a, pv, _ = _run_batch(solver_cls, mix, 10, mode=mode, device_loop=True, zone_cap=cap, pair_capacity=pc,
                              small_sort=small)
        b, _, _ = _run_batch(solver_cls, mix, 10, mode=mode, device_loop=False, zone_cap=cap)
        zone_steps = capped = 0
        for k, (u, w) in enumerate(zip(a, b)):
            capped += int((u["status"] != 0).sum())
            for key in ("x", "v", "hc", "hcol", "status"):
                assert np.array_equal(u[key], w[key]), (k, key)
            for i in range(len(mix)):
                assert np.array_equal(u["kinds"][i], w["kinds"][i]), (k, i)
                zone_steps += int((np.asarray(u["kinds"][i]) == 2).any())
            assert np.array_equal(zone_labels(u["zones"]), zone_labels(w["zones"])), k
            # the device loop's later passes test only pairs with a point the
            # previous pass touched: fewer candidate pairs and visits, the
            # same hits and contacts
            for c in ("passes", "ccd_passes", "zone_passes", "hit_pairs", "contacts"):
                assert u["counters"][c] == w["counters"][c], (k, c)
            assert u["counters"]["visits"] <= w["counters"]["visits"], k
            assert u["counters"]["loop_passes"] > 0 and w["counters"]["loop_passes"] == 0, k
        if cap is not None:
            assert zone_steps > 0 and capped > 0


def test_loop_stage_marks_change_nothing(solver_cls):
    # profiling level 2 puts boundary kernels between the stages of every
    # pass of the loop graph; results are unchanged and every pass is split
    mix = _contact_sample()
    ref, _, _ = _run_batch(solver_cls, mix, 3, mode=1)
    b = solver_cls(0)
    b.assembleBatch(mix)
    b.setMode(1)
    b.setProfiling(2)
    x = np.concatenate([s.x for s in mix])
    v = np.concatenate([s.v for s in mix])
    hc = np.zeros(len(x), np.uint8)
    dt = np.concatenate([np.full(s.nv, s.params["dt"]) for s in mix])[:, None]
    for r in ref:
        xo, vo, ho, hcol = b.resolveCollisionBatch(x, x + dt * v, v, hc)
        assert np.array_equal(xo, r["x"]) and np.array_equal(vo, r["v"]) and np.array_equal(ho, r["hc"])
        x, v, hc = xo, vo, ho
    prof = b.profile()
    loop_passes = sum(r["counters"]["loop_passes"] for r in ref)
    assert loop_passes > 0
    assert prof["loop_traverse"][1] == prof["loop_end"][1] >= loop_passes
    loop_ms = sum(prof[k][0] for k in prof if k.startswith("loop_"))
    assert 0 < loop_ms <= prof["detect_loop"][0] * 1.05
    b.close()


@pytest.mark.parametrize("mode", [0, 1], ids=["plain", "mixed"])
def test_pruned_walks_agree(solver_cls, mode):
    # the device loop's pruned passes walk each dirty element's scene with
    # one warp and a shared-memory stack, or with one thread along the
    # ropes: the same candidate pairs, so the same counts and results
    mix = _contact_sample()
    a, _, _ = _run_batch(solver_cls, mix, 8, mode=mode, zone_cap=3, pruned_warp=True)
    b, _, _ = _run_batch(solver_cls, mix, 8, mode=mode, zone_cap=3, pruned_warp=False)
    for k, (u, w) in enumerate(zip(a, b)):
        for key in ("x", "v", "hc", "hcol", "status"):
            assert np.array_equal(u[key], w[key]), (k, key)
        for c in ("passes", "candidate_pairs", "visits", "hit_pairs", "contacts", "pruned_queries"):
            assert u["counters"][c] == w["counters"][c], (k, c)
    assert sum(u["counters"]["pruned_queries"] for u in a) > 0


@pytest.mark.parametrize("device_loop", [True, False])
def test_refit_walks_agree(solver_cls, device_loop):
    # the hierarchy refit with one acquire-release arrival per level, ending
    # at each scene's root, writes the node boxes the fenced walk to the top
    # writes: the same pairs, counts and results, through the device loop
    # and through the host's passes
    mix = _contact_sample()
    a, _, _ = _run_batch(solver_cls, mix, 8, mode=1, zone_cap=3, device_loop=device_loop, refit_up=True)
    b, _, _ = _run_batch(solver_cls, mix, 8, mode=1, zone_cap=3, device_loop=device_loop, refit_up=False)
    for k, (u, w) in enumerate(zip(a, b)):
        for key in ("x", "v", "hc", "hcol", "status"):
            assert np.array_equal(u[key], w[key]), (k, key)
        for c in ("passes", "candidate_pairs", "visits", "hit_pairs", "contacts"):
            assert u["counters"][c] == w["counters"][c], (k, c)


def test_robust_roots_change_nothing(solver_cls):
    # the mixed sub-tests skip the correctly rounded recomputation of roots
    # well inside the window at which the test misses with a margin; every
    # result is the same as with every near root formed again
    for mix, steps in ((_contact_sample(), 6), ([scenes.large(n=65)], 8)):
        a, _, _ = _run_batch(solver_cls, mix, steps, mode=1, zone_cap=50, robust_roots=True)
        b, _, _ = _run_batch(solver_cls, mix, steps, mode=1, zone_cap=50, robust_roots=False)
        cr_a = cr_b = 0
        for k, (u, w) in enumerate(zip(a, b)):
            for key in ("x", "v", "hc", "hcol", "status"):
                assert np.array_equal(u[key], w[key]), (k, key)
            for c in ("passes", "candidate_pairs", "visits", "hit_pairs", "contacts", "fp64_subtests"):
                assert u["counters"][c] == w["counters"][c], (k, c)
            cr_a += u["counters"]["cr_roots"]
            cr_b += w["counters"]["cr_roots"]
        assert cr_b > 0 and cr_a <= cr_b, (cr_a, cr_b)
        print("correctly rounded cubics with and without the skip:", cr_a, cr_b)


def test_zone_cta_solve_agrees(solver_cls):
    # zones of 16+ members solved by one CTA each instead of one warp each:
    # the same sums in the same order, so the same bits
    mix = _contact_sample()
    a, _, _ = _run_batch(solver_cls, mix, 8, mode=1, zone_cap=50)
    b, _, _ = _run_batch(solver_cls, mix, 8, mode=1, zone_cap=50, zone_cta_min=16)
    zone_steps = 0
    for k, (u, w) in enumerate(zip(a, b)):
        for key in ("x", "v", "hc", "hcol", "status", "zones"):
            assert np.array_equal(u[key], w[key]), (k, key)
        zone_steps += u["counters"]["zone_passes"] > 0
    assert zone_steps > 0


@pytest.mark.parametrize("device_loop", [True, False])
def test_merged_subtests_agree(solver_cls, device_loop):
    # the FP64 sub-tests of both kinds in one launch (a warp each in small
    # passes) and one launch per kind (a thread each): the same tests on the
    # same records, so the same counts and bits
    mix = _contact_sample()
    a, _, _ = _run_batch(solver_cls, mix, 8, mode=1, zone_cap=3, device_loop=device_loop, sub_merge=True)
    b, _, _ = _run_batch(solver_cls, mix, 8, mode=1, zone_cap=3, device_loop=device_loop, sub_merge=False)
    for k, (u, w) in enumerate(zip(a, b)):
        for key in ("x", "v", "hc", "hcol", "status"):
            assert np.array_equal(u[key], w[key]), (k, key)
        for c in ("passes", "visits", "hit_pairs", "contacts", "fp64_subtests"):
            assert u["counters"][c] == w["counters"][c], (k, c)


def test_zone_warp_solve_for_few_zones_agrees(solver_cls):
    # zones of 2-15 members solved one thread each (ZONE_FEW 0), one warp
    # each in every pass (a large ZONE_FEW) and the default (a warp each
    # where a pass has at most 1,024 zones): the same operations in the same
    # order - the warps' sin and cos on two lanes equal one thread's sincos -
    # so the same bits
    for mix in (_contact_sample(), [scenes.large(n=65)]):
        runs = [_run_batch(solver_cls, mix, 8, mode=1, zone_cap=50, zone_few=f)[0] for f in (0, 1 << 30, None)]
        zone_steps = 0
        for k in range(8):
            for other in runs[1:]:
                for key in ("x", "v", "hc", "hcol", "status", "zones"):
                    assert np.array_equal(runs[0][k][key], other[k][key]), (k, key)
            zone_steps += runs[0][k]["counters"]["zone_passes"] > 0
        assert zone_steps > 0


def test_zone_replay_in_shared_memory_agrees(solver_cls):
    # every final zone's unions replayed by a CTA in a shared-memory table
    # (threshold 1), by one thread from global memory (0), and the default:
    # the same unions in the same order, so the same zones and bits
    for mix in (_contact_sample(), [scenes.large(n=65)]):
        runs = [_run_batch(solver_cls, mix, 8, mode=1, zone_cap=50, replay_cta_min=m)[0] for m in (None, 1, 0)]
        unions = 0
        for k in range(8):
            for other in runs[1:]:
                for key in ("x", "v", "hc", "hcol", "status", "zones"):
                    assert np.array_equal(runs[0][k][key], other[k][key]), (k, key)
            unions += runs[0][k]["counters"]["zone_unions"]
        assert unions > 0
