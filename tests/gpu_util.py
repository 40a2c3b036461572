"""Helpers shared by the GPU parity tests."""
import hashlib

import numpy as np

from collision_gb300 import scenes


def scene_from_golden(g):
    bodies = {}
    if "scene_body_surf" in g:
        for i, sid in enumerate(g["scene_body_surf"].tolist()):
            bodies[int(sid)] = dict(mass=float(g["scene_body_mass"][i]), com=g["scene_body_com"][i].copy(),
                                    comv=g["scene_body_comv"][i].copy())
    return scenes.Scene("golden", g["scene_x"], g["scene_v"], g["scene_fixed"], g["scene_tris"],
                        g["scene_tri_surf"], g["scene_tri_rest"], g["scene_bonds"], g["scene_bond_curve"],
                        g["scene_bond_rest"], g["scene_domain"],
                        dict(zip(scenes.PARAM_NAMES, g["scene_params"].tolist())), bodies)


def golden_inputs(g, sc, step):
    """(x_old, x_cand, vel, has_collsn) of a fixture's step: stored, or for a
    chained fixture the previous step's outputs (the scene's state at step 0)
    with candidate positions x + dt*v."""
    if "x_old" in g:
        return g["x_old"][step], g["x_cand"][step], g["vel_in"][step], g["hc_in"][step]
    if step == 0:
        x, v, hc = sc.x, sc.v, np.zeros(sc.nv, np.uint8)
    else:
        x, v, hc = g["x"][step - 1], g["vel"][step - 1], g["hc"][step - 1]
    return x, scenes.candidate(sc, x, v), v, hc


def record_sha(rec11: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(rec11, dtype="<i4").tobytes()).hexdigest()


def rel_err(a, b):
    """Norm-wise relative difference: max |a-b| over max(max |b|, 1)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.size == 0:
        return 0.0
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1.0))


def zone_labels(zone_root):
    zr = np.asarray(zone_root)
    mins = {}
    for i, r in enumerate(zr):
        mins[r] = min(mins.get(r, i), i)
    return np.array([mins[r] for r in zr], dtype=np.int32)
