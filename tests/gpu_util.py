"""Helpers shared by the GPU parity tests."""
import hashlib

import numpy as np

from collision_gb300 import scenes


def scene_from_golden(g):
    return scenes.Scene("golden", g["scene_x"], g["scene_v"], g["scene_fixed"], g["scene_tris"],
                        g["scene_tri_surf"], g["scene_tri_rest"], g["scene_bonds"], g["scene_bond_curve"],
                        g["scene_bond_rest"], g["scene_domain"],
                        dict(zip(scenes.PARAM_NAMES, g["scene_params"].tolist())))


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
