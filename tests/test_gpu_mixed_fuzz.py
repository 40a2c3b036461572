"""Mixed-precision filters against plain FP64 on near-contact configurations.

Thousands of two-element scenes (triangle-triangle, triangle-bond,
bond-bond) are placed at distances around the thickness h, some coplanar
with in-plane offsets, some nearly parallel, with relative velocities that
cross within dt, and resolved in one batch in both arithmetic modes. The
FP32 filters may only skip sub-tests that cannot hit, so every output must
be bit-identical between the modes; the cases are checked to contain many
hits so that a filter rejecting a real contact would show.
"""
import numpy as np
import pytest

from collision_gb300 import scenes

pytestmark = pytest.mark.gpu


def _rand_unit(rng):
    v = rng.normal(size=3)
    return v / np.linalg.norm(v)


def _frame(rng):
    a = _rand_unit(rng)
    b = np.cross(a, _rand_unit(rng))
    b /= np.linalg.norm(b)
    return a, b, np.cross(a, b)


def _tri(rng, size):
    u, w, _ = _frame(rng)
    p0 = np.zeros(3)
    p1 = size * (0.6 + 0.8 * rng.random()) * u
    p2 = size * (0.6 + 0.8 * rng.random()) * (np.cos(rng.uniform(0.3, 2.6)) * u + np.sin(rng.uniform(0.3, 2.6)) * w)
    return np.stack([p0, p1, p2])


def _case(rng, kind, h, dt):
    size = 10 ** rng.uniform(-2.5, -0.5)
    style = rng.integers(0, 4)
    A = _tri(rng, size) if kind != 2 else _tri(rng, size)[:2]
    if style == 0:
        # B near a random point of A, offset along a random direction by ~h
        B = (_tri(rng, size) if kind == 0 else _tri(rng, size)[:2])
        anchor = A.mean(axis=0) + rng.uniform(-0.5, 0.5) * (A[1] - A[0])
        B = B - B[rng.integers(0, len(B))] + anchor + _rand_unit(rng) * h * rng.uniform(0.2, 3.0)
    elif style == 1:
        # coplanar with A, shifted in-plane by a fraction of its size (flat cloth)
        n = np.cross(A[1] - A[0], (A[2] if len(A) == 3 else A[0] + _rand_unit(rng)) - A[0])
        n /= np.linalg.norm(n)
        d = _rand_unit(rng)
        d -= d.dot(n) * n
        d /= np.linalg.norm(d)
        B = A[[1, 2, 0]] if kind == 0 else A[:2]
        B = B + d * size * rng.uniform(0.0, 1.2) + n * h * rng.uniform(-0.3, 0.3)
        if kind == 1:
            B = A[:2] + d * size * rng.uniform(0.0, 1.2)
    elif style == 2:
        # nearly parallel edges
        e = A[1] - A[0]
        tw = _rand_unit(rng) * 1e-6 * size * rng.random()
        B = np.stack([A[0] + tw, A[1] - tw]) + _rand_unit(rng) * h * rng.uniform(0.0, 2.0)
        if kind == 0:
            B = np.vstack([B, A[2] + _rand_unit(rng) * size])
        e = e
    else:
        # B crosses A's plane within the step
        B = (_tri(rng, size) if kind == 0 else _tri(rng, size)[:2])
        B = B - B.mean(axis=0) + A.mean(axis=0) + _rand_unit(rng) * size * rng.uniform(0.05, 0.5)
    if kind == 1:
        A, B = (A, B[:2]) if len(A) == 3 else (B, A)
    va = rng.normal(size=3) * 0.1
    vb = va + _rand_unit(rng) * rng.uniform(0.0, 3.0) * size / dt * rng.choice([0.0, 0.01, 0.3, 1.0])
    VA = np.tile(va, (len(A), 1)) + rng.normal(size=(len(A), 3)) * 1e-3
    VB = np.tile(vb, (len(B), 1)) + rng.normal(size=(len(B), 3)) * 1e-3
    x = np.vstack([A, B]) + rng.uniform(-1, 1, size=3)
    v = np.vstack([VA, VB])
    na = len(A)
    tris, bonds = [], []
    for idx, n_pts in ((0, na), (na, len(B))):
        if n_pts == 3:
            tris.append([idx, idx + 1, idx + 2])
        else:
            bonds.append([idx, idx + 1])
    tris = np.array(tris, np.int32).reshape(-1, 3)
    bonds = np.array(bonds, np.int32).reshape(-1, 2)
    tri_rest = np.array([[np.linalg.norm(x[t[(j + 1) % 3]] - x[t[j]]) for j in range(3)] for t in tris]).reshape(-1, 3)
    bond_rest = np.array([np.linalg.norm(x[b[1]] - x[b[0]]) for b in bonds])
    fixed = np.zeros(len(x), np.uint8)
    if rng.random() < 0.2 and len(tris):
        fixed[tris[0]] = 1
    dom = np.concatenate([x.min(0) - 10, x.max(0) + 10])
    return scenes.Scene(f"fuzz{kind}{style}", x, v, fixed, tris, np.arange(len(tris), dtype=np.int32),
                        tri_rest, bonds, np.zeros(len(bonds), np.int32), bond_rest, dom,
                        dict(scenes.DEFAULTS, dt=dt, thickness=h))


def _resolvable(sc, nsteps):
    """The CPU oracle resolves nsteps steps of the scene. Some random
    configurations reach the reference's exits (a degenerate contact normal,
    dcollid3d.cpp:905-909, 756-760); a batch stops at the first scene that
    does, so such cases are left out."""
    from oracle.ccopy import OracleSolver
    o = OracleSolver(sc, record=0)
    x, v, hc = sc.x, sc.v, np.zeros(sc.nv, np.uint8)
    for _ in range(nsteps):
        r = o.step(x, x + sc.params["dt"] * v, v, hc)
        if r["rc"] != 0:
            return False
        x, v, hc = r["x"], r["v"], r["has_collsn"]
    return True


def _cases(n, seed, nsteps, h=1e-3, dt=1e-3):
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        sc = _case(rng, int(rng.integers(0, 3)), h, dt)
        if _resolvable(sc, nsteps):
            out.append(sc)
    return out


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_mixed_equals_plain_near_contact(seed):
    from collision_gb300.solver import CollisionSolver3d
    mix = _cases(3000, seed, 3)
    x = np.concatenate([s.x for s in mix])
    v = np.concatenate([s.v for s in mix])
    dt = np.concatenate([np.full((s.nv, 1), s.params["dt"]) for s in mix])
    out = {}
    for mode in (0, 1):
        b = CollisionSolver3d(0)
        b.assembleBatch(mix)
        b.setMode(mode)
        xs, vs, hc = x, v, np.zeros(len(x), np.uint8)
        res = []
        for _ in range(3):
            xo, vo, ho, hcol = b.resolveCollisionBatch(xs, xs + dt * vs, vs, hc)
            res.append((xo, vo, ho, hcol, b.counters()))
            xs, vs, hc = xo, vo, ho
        out[mode] = res
        b.close()
    for k in range(3):
        p, m = out[0][k], out[1][k]
        assert np.array_equal(p[0], m[0]), k
        assert np.array_equal(p[1], m[1]), k
        assert np.array_equal(p[2], m[2]), k
        assert np.array_equal(p[3], m[3]), k
        assert p[4]["hit_pairs"] == m[4]["hit_pairs"]
        assert p[4]["contacts"] == m[4]["contacts"]
    # the cases must exercise contacts, and the filters must skip work
    assert out[0][0][4]["contacts"] > 500
    assert out[1][0][4]["fp64_subtests"] < out[0][0][4]["fp64_subtests"]
