"""Small seeded scenes for the golden fixtures and the oracle pin.

Each case is (scene factory, number of steps). They are sized so the
reference finishes each in well under a second and together they reach every
branch the workloads use: point-triangle and edge-edge proximity and CCD,
tri-bond and bond-bond pairs, up to five CCD passes, impact zones, strain
limiting, tree rebuilds, a pinned cloth point (mixed rigidity within one
surface) and an active domain clamp.
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


CASES = {
    "sphere9": (_sphere9, 10),
    "sphere12_fast": (_sphere12_fast, 8),
    "strings_box": (_strings_box, 10),
    "folded17": (_folded17, 10),
    "pinned_domain": (_pinned_domain, 8),
}
