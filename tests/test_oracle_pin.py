"""The CPU oracle (oracle/cc_oracle.c) reproduces the reference bit for bit.

The golden fixtures were produced by the reference's own solver sources
(tests/golden/make_golden.py). For every step the oracle is fed the same
inputs and must return identical positions, velocities, collision flags,
impact-zone partition, pass sequence, narrow-phase visit record (order,
orientation and status of every call, by SHA-256) and hit list. The
oracle's build with correctly rounded acos/cos/sin/pow (CCO_CRMATH), which
the GPU parity runs use to tell glibc's misroundings apart, must give the
same on every golden step: none of them depends on such a misrounding.
"""
import glob
import hashlib
import os

import numpy as np
import pytest

from collision_gb300 import scenes
from oracle.ccopy import OracleSolver, REC_PAIRS, zone_labels
from tests.gpu_util import golden_inputs, scene_from_golden

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def test_golden_present():
    assert len(GOLDEN) >= 12


@pytest.mark.parametrize("crmath", [False, True], ids=["libm", "crmath"])
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_matches_reference_golden(path, crmath):
    g = np.load(path)
    sc = scene_from_golden(g)
    o = OracleSolver(sc, record=REC_PAIRS, crmath=crmath)
    nsteps = len(g["x"])
    for step in range(nsteps):
        out = o.step(*golden_inputs(g, sc, step))
        assert out["rc"] == 0
        assert np.array_equal(out["x"], g["x"][step]), f"positions differ at step {step}"
        assert np.array_equal(out["v"], g["vel"][step]), f"velocities differ at step {step}"
        assert np.array_equal(out["has_collsn"], g["hc"][step])
        assert out["has_collision"] == g["has_collision"][step]
        assert np.array_equal(zone_labels(out["zone_root"]), g["zones"][step])
        kinds = g["pass_kinds"][g["pass_kinds"][:, 0] == step][:, 1]
        assert np.array_equal(o.passes(), kinds)
        p = o.pairs()
        assert len(p) == g["npairs"][step]
        assert hashlib.sha256(np.ascontiguousarray(p, dtype="<i4").tobytes()).hexdigest() == \
            str(g["pair_sha"][step])
        hits = g["hits"][g["hits"][:, 0] == step][:, 1:]
        assert np.array_equal(p[p[:, 4] != 0], hits)
        for i, sid in enumerate(sorted(sc.bodies)):
            com, comv = o.body(sid)
            assert np.array_equal(com, g["body_com"][step][i]), f"body {sid} centre of mass, step {step}"
            assert np.array_equal(comv, g["body_comv"][step][i]), f"body {sid} velocity, step {step}"
    o.close()


def test_oracle_rejects_bad_vertex_index():
    sc = scenes.cloth_on_sphere(n=4, sub=1, side=0.2)
    sc.tris = sc.tris.copy()
    sc.tris[0, 0] = sc.nv + 5
    with pytest.raises(ValueError):
        OracleSolver(sc)


def test_oracle_empty_mesh_passes_through():
    # The reference dereferences an empty tree here; the oracle returns the
    # candidate positions untouched.
    sc = scenes.cloth_on_sphere(n=4, sub=1, side=0.2)
    sc.tris = np.zeros((0, 3), np.int32)
    sc.tri_surf = np.zeros(0, np.int32)
    sc.tri_rest = np.zeros((0, 3))
    o = OracleSolver(sc)
    xc = scenes.candidate(sc, sc.x, sc.v)
    out = o.step(sc.x, xc, sc.v, np.zeros(sc.nv, np.uint8))
    assert out["rc"] == 0
    assert np.array_equal(out["x"], xc)
