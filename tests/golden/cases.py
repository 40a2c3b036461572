"""Small seeded scenes for the golden fixtures and the oracle pin.

Each case is (scene factory, number of steps). They are sized so the
reference finishes each in well under a second and together they reach every
branch the workloads use: point-triangle and edge-edge proximity and CCD,
tri-bond and bond-bond pairs, up to five CCD passes, impact zones, strain
limiting, tree rebuilds, a pinned cloth point (mixed rigidity within one
surface), an active domain clamp, movable rigid bodies (body-body, body-fixed
and cloth-body contacts) and the reference's six input decks.
"""
from __future__ import annotations

import numpy as np

from collision_gb300 import scenes


def _sphere9():
    return scenes.cloth_on_sphere(n=9, z=0.2525, radius=0.25, sub=2, side=0.3)


def _sphere12_fast():
    # 3 m/s with friction 0.3: five CCD passes, then impact zones
    return scenes.cloth_on_sphere(n=12, z=0.252, radius=0.25, sub=2, side=0.4, mu=0.3,
                                  speed=3.0, seed=2)


def _strings_box():
    return scenes.strings(nstr=8, nseg=60, seglen=4e-3, seed=1, box_lo=(-0.2, -0.2, -0.05),
                          box_hi=(0.2, 0.2, 0.049), z_range=(0.0505, 0.06), volume_z=(0.05, 0.07),
                          speed=1.0, h=2e-3)


def _folded17():
    return scenes.folded_cloth(n=17, dt=5e-4, h=5e-3, seed=3, vscale=20.0)


def _pinned_domain():
    sc = scenes.cloth_on_sphere(n=10, z=0.252, radius=0.25, sub=2, side=0.4, mu=0.3, speed=2.0, seed=5)
    sc.fixed[0] = 1
    sc.v[0] = 0.0
    sc.domain = np.array([-0.19, -0.19, 0.0, 0.19, 0.19, 1.0])
    return sc


def _shift_part(sc, lo, hi, d):
    """Moves points [lo, hi) by d (breaks an exact alignment of two meshes
    that would reach the reference's degenerate-normal exit)."""
    sc.x[lo:hi] += np.asarray(d, dtype=np.float64)
    for b in sc.bodies.values():
        b["com"] = b["com"] + np.asarray(d, dtype=np.float64) if lo == 0 else b["com"]
    return sc


def _rigid_bodies():
    # two movable spheres (masses 2 and 1) meeting each other and a fixed
    # box, with a small cloth falling onto the first
    a, at = scenes.icosphere(1, 0.05, center=(0.0123, 0.0071, 0.0515))
    b, bt = scenes.icosphere(1, 0.05, center=(0.1135, 0.0071, 0.0515))
    bp, bx = scenes.box_mesh((-0.2, -0.2, -0.05), (0.25, 0.2, 0.0))
    c, ct = scenes.grid_cloth(5, 0.1, 0.1035, center=(0.012, 0.007))
    parts = [(a, at, np.tile([0.0, 0.0, -0.5], (len(a), 1)), 2),
             (b, bt, np.tile([-0.5, 0.0, 0.0], (len(b), 1)), 2),
             (bp, bx, np.zeros_like(bp), True),
             (c, ct, np.tile([0.0, 0.0, -0.8], (len(c), 1)), False)]
    return scenes.assemble("rigid_bodies", parts, dict(dt=1e-3, thickness=1e-3, lam=0.1),
                           masses={0: 2.0, 1: 1.0})


def _sphere12_movable():
    # sphere12_fast with the sphere a movable body of mass 0.5: impact-zone
    # passes (steps 5-7) with a body among the zones
    sc = _sphere12_fast()
    pts = np.unique(sc.tris[sc.tri_surf == 1])
    sc.fixed[pts] = 2
    sc.bodies = {1: dict(mass=0.5, com=sc.x[pts].mean(axis=0), comv=np.zeros(3))}
    return sc


def _deck_ball_plane():
    # a movable sphere rising into a free plate
    return _shift_part(scenes.deck("ball_plane", advance=0.021, sub=2, cells=20), 0, 162, (0.0013, 0.0007, 0.0))


def _deck_string_slide():
    # a string sliding onto a movable box
    return scenes.deck("string_slide", advance=0.0433, cells=20)


def _deck_ball_ball():
    return scenes.deck("ball_ball", advance=0.155, sub=2, cells=20)


def _deck_string_box():
    sc = scenes.deck("string_box", advance=0.0953, cells=20)
    return _shift_part(sc, sc.nv - (sc.nb + 1), sc.nv, (0.0011, 0.0003, 0.00017))


def _deck_string_string():
    return scenes.deck("string_string", advance=0.022, cells=20)


def _deck_box_boundary():
    # a movable box heading for the domain's floor (the clamp leaves movable
    # points alone, dcollid.cpp:123)
    return scenes.deck("box_boundary", advance=0.02, cells=20)


CASES = {
    "sphere9": (_sphere9, 10),
    "sphere12_fast": (_sphere12_fast, 8),
    "strings_box": (_strings_box, 10),
    "folded17": (_folded17, 10),
    "pinned_domain": (_pinned_domain, 8),
    "rigid_bodies": (_rigid_bodies, 8),
    "sphere12_movable": (_sphere12_movable, 8),
    "deck_ball_plane": (_deck_ball_plane, 8),
    "deck_string_slide": (_deck_string_slide, 10),
    "deck_ball_ball": (_deck_ball_ball, 8),
    "deck_string_box": (_deck_string_box, 8),
    "deck_string_string": (_deck_string_string, 8),
    "deck_box_boundary": (_deck_box_boundary, 8),
}
# Cases whose fixtures keep only the outputs of each step: the inputs of step
# k+1 are the outputs of step k (candidate positions x + dt*v, as the host
# loop forms them), and step 0 starts from the scene.
CHAINED = {"rigid_bodies", "sphere12_movable", "deck_ball_plane", "deck_string_slide", "deck_ball_ball", "deck_string_box",
           "deck_string_string", "deck_box_boundary"}
