"""Lockstep runs of the GPU solver beside the oracle (test infrastructure).

Every step, the same inputs go to
  - the oracle (oracle/cc_oracle.c, bit-exact to the reference compiled from
    its sources, glibc's acos/cos/sin/pow),
  - the oracle's CCO_CRMATH build (the same algorithm with correctly rounded
    acos/cos/sin/pow, as the GPU path evaluates them),
  - the GPU solver(s),
and the step's outputs are compared: pass sequence, impact-zone partition,
has_collsn, hasCollision, positions and velocities bit for bit, and (with
recording) the full narrow-phase visit record by SHA-256. A step is "exact"
when the GPU equals the oracle, a "glibc residual" when it differs from the
oracle but equals the correctly rounded build (glibc misrounded an argument
that decided the result; the difference is measured), and a failure
otherwise. The next step's inputs are the oracle's outputs, so every step is
compared from the same state.
"""
from __future__ import annotations

import dataclasses
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from collision_gb300 import scenes
from collision_gb300.solver import ordered_visits
from oracle.ccopy import REC_PAIRS, OracleSolver
from tests.gpu_util import record_sha, zone_labels

ORACLE_ITER_CAP = -3


@dataclasses.dataclass
class Tally:
    steps: int = 0
    exact: int = 0
    glibc: int = 0            # steps explained by glibc's rounding
    contact_steps: int = 0    # steps with a CCD pass that hit (more than two passes)
    zone_steps: int = 0       # steps with an impact-zone pass
    max_abs_x: float = 0.0    # over glibc-residual steps: GPU vs oracle
    max_rel_x: float = 0.0    # per element, |d| / max(|ref|, 1e-6)
    max_abs_v: float = 0.0
    max_rel_v: float = 0.0
    cr_roots: int = 0         # GPU cubics re-rooted with the correctly rounded functions
    capped: int = 0           # scene-steps stopped at the zone cap (both sides)
    missed: int = 0           # pairs the exact CCD re-check finds after exact steps (GPU = oracle)

    def note(self, kinds):
        k = np.asarray(kinds)
        self.contact_steps += int(len(k) > 2)
        self.zone_steps += int((k == 2).any())

    def merge(self, o: "Tally"):
        for f in dataclasses.fields(self):
            a, b = getattr(self, f.name), getattr(o, f.name)
            setattr(self, f.name, max(a, b) if f.name.startswith("max_") else a + b)


def _rel(a, b):
    d = np.abs(np.asarray(a) - np.asarray(b))
    if d.size == 0:
        return 0.0, 0.0
    return float(d.max()), float((d / np.maximum(np.abs(b), 1e-6)).max())


def fast_forward(sc, nsteps):
    """The scene's state after nsteps oracle steps from its initial state."""
    o = OracleSolver(sc, record=0)
    x, v, hc = sc.x.copy(), sc.v.copy(), np.zeros(sc.nv, np.uint8)
    for _ in range(nsteps):
        r = o.step(x, scenes.candidate(sc, x, v), v, hc)
        assert r["rc"] == 0
        x, v, hc = r["x"], r["v"], r["has_collsn"]
    o.close()
    return x, v, hc


class _Ref:
    """The two oracle builds of one scene, stepped together."""

    def __init__(self, sc, record, zone_cap):
        self.o = OracleSolver(sc, record=REC_PAIRS if record else 0)
        self.c = OracleSolver(sc, record=REC_PAIRS if record else 0, crmath=True)
        if zone_cap is not None:
            self.o.set_zone_cap(zone_cap)
            self.c.set_zone_cap(zone_cap)
        self.record = record

    def view(self, solver, r):
        return dict(x=r["x"], v=r["v"], hc=r["has_collsn"], hcol=bool(r["has_collision"]),
                    kinds=solver.passes(), zones=zone_labels(r["zone_root"]),
                    sha=record_sha(solver.pairs()) if self.record else None, rc=r["rc"])

    def close(self):
        self.o.close()
        self.c.close()


def _match(g, ref):
    return (np.array_equal(g["kinds"], ref["kinds"]) and np.array_equal(g["zones"], ref["zones"]) and
            np.array_equal(g["hc"], ref["hc"]) and g["hcol"] == ref["hcol"] and
            np.array_equal(g["x"], ref["x"]) and np.array_equal(g["v"], ref["v"]) and
            (g["sha"] is None or g["sha"] == ref["sha"]))


def _assess(t: Tally, g, ro, rc, where):
    """Count a step exact or glibc-residual, or fail with the differences."""
    if _match(g, ro):
        t.exact += 1
        return
    if _match(g, rc):
        t.glibc += 1
        ax, rx = _rel(g["x"], ro["x"])
        av, rv = _rel(g["v"], ro["v"])
        t.max_abs_x, t.max_rel_x = max(t.max_abs_x, ax), max(t.max_rel_x, rx)
        t.max_abs_v, t.max_rel_v = max(t.max_abs_v, av), max(t.max_rel_v, rv)
        return
    parts = []
    for k in ("kinds", "zones", "hc", "hcol", "sha"):
        if not np.array_equal(np.asarray(g[k]), np.asarray(ro[k])):
            parts.append(k)
    raise AssertionError(f"{where}: GPU differs from the oracle ({', '.join(parts) or 'state'}; "
                         f"x {_rel(g['x'], ro['x'])}, v {_rel(g['v'], ro['v'])}) and from its correctly "
                         f"rounded build (x {_rel(g['x'], rc['x'])})")


def run_scene(solver_cls, sc, nsteps, start=None, record=True, label="") -> Tally:
    """One scene: the plain FP64 GPU path (recording visits when `record`)
    and the mixed-precision path (split narrow phase, no recording) against
    both oracle builds, step by step."""
    x, v, hc = start if start is not None else (sc.x.copy(), sc.v.copy(), np.zeros(sc.nv, np.uint8))
    ref = _Ref(sc, record, None)
    plain, mixed = solver_cls(0), solver_cls(0)
    plain.assembleFromScene(sc)
    plain.setRecording(record)
    mixed.assembleFromScene(sc)
    mixed.setMode(1)
    t = Tally()
    with ThreadPoolExecutor(2) as ex:
        for step in range(nsteps):
            xc = scenes.candidate(sc, x, v)
            fo = ex.submit(ref.o.step, x, xc, v, hc)
            fc = ex.submit(ref.c.step, x, xc, v, hc)
            xp, vp, hp = plain.resolveCollision(x, xc, v, hc)
            g = dict(x=xp, v=vp, hc=hp, hcol=plain.hasCollision(), kinds=plain.passKinds(),
                     zones=zone_labels(plain.zoneRoots()),
                     sha=record_sha(ordered_visits(plain.visits())) if record else None)
            t.cr_roots += plain.counters()["cr_roots"]
            xm, vm, hm = mixed.resolveCollision(x, xc, v, hc)
            where = f"{label} step {step}"
            assert np.array_equal(xm, xp) and np.array_equal(vm, vp) and np.array_equal(hm, hp), \
                f"{where}: mixed precision differs from plain FP64"
            assert np.array_equal(mixed.passKinds(), g["kinds"]), f"{where}: mixed pass sequence"
            assert np.array_equal(zone_labels(mixed.zoneRoots()), g["zones"]), f"{where}: mixed zones"
            r, q = fo.result(), fc.result()
            assert r["rc"] == 0 and q["rc"] == 0, (where, r["rc"], q["rc"])
            ro, rc = ref.view(ref.o, r), ref.view(ref.c, q)
            _assess(t, g, ro, rc, where)
            t.note(g["kinds"])
            t.steps += 1
            x, v, hc = r["x"], r["v"], r["has_collsn"]
    plain.close()
    mixed.close()
    ref.close()
    return t


def run_batch(solver_cls, scs, nsteps, mode=1, zone_cap=200, threads=16, label="") -> Tally:
    """Scenes resolved together in one batch (the batched path; mixed
    precision by default, no recording) against both oracle builds of every
    scene. A scene that reaches the zone cap on both sides is left out from
    then on. After every step the exact CCD re-check runs on the GPU
    (cc_check_ccd) and on the oracle's CPU restatement of it, and on every
    scene whose step was exact the two must find the same pairs."""
    import torch
    b = solver_cls(0)
    b.assembleBatch(scs)
    b.setMode(mode)
    b.setZoneCap(zone_cap)
    pv, _ = b.sceneOffsets()
    refs = [_Ref(sc, False, zone_cap) for sc in scs]
    x = np.concatenate([sc.x for sc in scs])
    v = np.concatenate([sc.v for sc in scs])
    hc = np.zeros(len(x), np.uint8)
    dt = np.concatenate([np.full((sc.nv, 1), sc.params["dt"]) for sc in scs])
    live = [True] * len(scs)
    t = Tally()
    with ThreadPoolExecutor(threads) as ex:
        for step in range(nsteps):
            xc = x + dt * v
            jobs = []
            for i, sc in enumerate(scs):
                if not live[i]:
                    continue
                a, e = int(pv[i]), int(pv[i + 1])
                args = (x[a:e], xc[a:e], v[a:e], hc[a:e])
                jobs.append((i, ex.submit(refs[i].o.step, *args), ex.submit(refs[i].c.step, *args)))
            xo, vo, ho, hcol = b.resolveCollisionBatch(x, xc, v, hc)
            status = b.sceneStatus()
            roots = b.zoneRoots()
            kinds = [b.scenePassKinds(i) for i in range(len(scs))]
            _, missed = b.checkCCD(torch.tensor(x, device="cuda:0"), torch.tensor(xo, device="cuda:0"))
            x_in = x
            x, v, hc = xo.copy(), vo.copy(), ho.copy()
            for i, fo, fc in jobs:
                a, e = int(pv[i]), int(pv[i + 1])
                r, q = fo.result(), fc.result()
                where = f"{label} step {step} scene {i}"
                if r["rc"] == ORACLE_ITER_CAP:
                    assert status[i] == solver_cls.ITER_CAP, f"{where}: the oracle reached the zone cap, GPU not"
                    live[i] = False
                    b.setSceneEnabled(i, False)
                    t.capped += 1
                    continue
                assert r["rc"] == 0 and q["rc"] == 0 and status[i] == 0, (where, r["rc"], q["rc"], status[i])
                g = dict(x=xo[a:e], v=vo[a:e], hc=ho[a:e], hcol=bool(hcol[i]), kinds=kinds[i],
                         zones=zone_labels(roots[a:e]), sha=None)
                exact_before = t.exact
                _assess(t, g, refs[i].view(refs[i].o, r), refs[i].view(refs[i].c, q), where)
                if t.exact > exact_before:
                    om = refs[i].o.check_ccd(x_in[a:e], r["x"])
                    assert om == missed[i], f"{where}: CCD re-check, GPU {missed[i]} vs oracle {om}"
                    t.missed += om
                t.note(g["kinds"])
                t.steps += 1
                x[a:e], v[a:e], hc[a:e] = r["x"], r["v"], r["has_collsn"]
            t.cr_roots += b.counters()["cr_roots"]
    b.close()
    for r in refs:
        r.close()
    return t
