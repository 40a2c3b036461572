"""Seeded synthetic scenes for the collision solver.

The reference publishes no dataset; its own decks (in-ball_ball, in-string_box,
...) need FronTier's surface builders, which are not available. These
generators make triangle/bond meshes with the shapes, sizes and velocity
distributions of the five workloads the solver is measured on:

  cloth_on_sphere   33x33 cloth (2,048 tris) at z=0.30 falling at (0,0,-1)+-0.01
                    onto a fixed icosphere r=0.25 (642 verts / 1,280 tris)
  folded_cloth      129x129 sinusoidal sheet (32,768 tris) driven by -2*grad(phi)
  strings           64 random-walk strings x 512 bonds of 2e-3 falling at
                    (0,0,-2) onto a fixed 0.4x0.4x0.1 box (12 tris)
  batched           256 cloth-on-obstacle scenes, 16..128 vertices per side
  large             1025x1025 cloth (2.1M tris) at (0,0,-10) onto a fixed
                    sub-5 icosphere (20,480 tris) r=0.3 next to a 12-tri box

Every array is in the layout the solver's C ABI takes: positions and
velocities (V,3) float64 point-major, triangles (T,3) int32 with a surface id
per triangle (contiguous runs), bonds (B,2) int32 with a curve id per bond
(contiguous runs), rest lengths = initial edge lengths (the reference's
side_length0 / length0, dcollid.cpp:513-516), point flags (V,) uint8 (1 fixed,
2 movable rigid body), and per movable surface its mass, centre of mass and
centre-of-mass velocity.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

# Solver parameter order used everywhere: dt, thickness, eps, k, m, lambda, cr.
PARAM_NAMES = ("dt", "thickness", "eps", "k", "m", "lam", "cr")
# Reference defaults (dcollid.cpp:28-35).
DEFAULTS = dict(dt=1e-3, thickness=1e-4, eps=1e-6, k=1000.0, m=0.01, lam=0.02, cr=0.0)


@dataclasses.dataclass
class Scene:
    name: str
    x: np.ndarray          # (V,3) float64 positions at the start of the step
    v: np.ndarray          # (V,3) float64 velocities
    fixed: np.ndarray      # (V,) uint8: 1 fixed obstacle point, 2 movable rigid body
    tris: np.ndarray       # (T,3) int32
    tri_surf: np.ndarray   # (T,) int32
    tri_rest: np.ndarray   # (T,3) float64
    bonds: np.ndarray      # (B,2) int32
    bond_curve: np.ndarray # (B,) int32
    bond_rest: np.ndarray  # (B,) float64
    domain: np.ndarray     # (6,) float64: lo xyz, hi xyz
    params: dict
    # movable rigid bodies: surface id -> dict(mass, com (3,), comv (3,))
    bodies: dict = dataclasses.field(default_factory=dict)

    @property
    def nv(self) -> int:
        return int(self.x.shape[0])

    @property
    def nt(self) -> int:
        return int(self.tris.shape[0])

    @property
    def nb(self) -> int:
        return int(self.bonds.shape[0])

    @property
    def ne(self) -> int:
        return self.nt + self.nb

    def param_vec(self) -> np.ndarray:
        return np.array([self.params[k] for k in PARAM_NAMES], dtype=np.float64)

    def copy(self) -> "Scene":
        return dataclasses.replace(
            self, **{f.name: (getattr(self, f.name).copy() if isinstance(getattr(self, f.name), np.ndarray)
                              else {k: (dict(v) if isinstance(v, dict) else v) for k, v in getattr(self, f.name).items()}
              if isinstance(getattr(self, f.name), dict)
                              else getattr(self, f.name))
                     for f in dataclasses.fields(self)})


# ---------------------------------------------------------------- primitives

def grid_cloth(n: int, side: float = 1.0, z: float = 0.0, center=(0.0, 0.0)):
    """n x n vertex sheet over [-side/2, side/2]^2, right-diagonal split:
    cell (i,j) -> (v00, v10, v11), (v00, v11, v01), cells row-major."""
    s = np.linspace(-0.5 * side, 0.5 * side, n)
    X, Y = np.meshgrid(s + center[0], s + center[1], indexing="xy")
    pts = np.stack([X.ravel(), Y.ravel(), np.full(n * n, z)], axis=1)
    i, j = np.meshgrid(np.arange(n - 1), np.arange(n - 1), indexing="xy")
    v00 = (j * n + i).ravel()
    v10 = v00 + 1
    v01 = v00 + n
    v11 = v01 + 1
    t1 = np.stack([v00, v10, v11], axis=1)
    t2 = np.stack([v00, v11, v01], axis=1)
    tris = np.stack([t1, t2], axis=1).reshape(-1, 3)
    return pts.astype(np.float64), tris.astype(np.int32)


def icosphere(sub: int, radius: float, center=(0.0, 0.0, 0.0)):
    """Subdivided icosahedron: 10*4^sub+2 vertices, 20*4^sub triangles."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0),
             (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
             (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
             (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
             (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    v = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in verts]
    for _ in range(sub):
        cache = {}
        nf = []

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = v[a] + v[b]
                v.append(m / np.linalg.norm(m))
                cache[key] = len(v) - 1
            return cache[key]

        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    pts = np.array(v) * radius + np.asarray(center, dtype=np.float64)
    return pts, np.array(faces, dtype=np.int32)


def box_mesh(lo, hi):
    """Axis-aligned box: 8 vertices, 12 triangles."""
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    pts = np.array([[lo[0] if (c & 1) == 0 else hi[0],
                     lo[1] if (c & 2) == 0 else hi[1],
                     lo[2] if (c & 4) == 0 else hi[2]] for c in range(8)])
    quads = [(0, 2, 3, 1), (4, 5, 7, 6), (0, 1, 5, 4), (2, 6, 7, 3), (0, 4, 6, 2), (1, 3, 7, 5)]
    tris = []
    for a, b, c, d in quads:
        tris += [(a, b, c), (a, c, d)]
    return pts, np.array(tris, dtype=np.int32)


def cuboid_mesh(center, edges, spacing):
    """Closed box surface, each face a grid of squares about `spacing` wide,
    split along one diagonal; outward-facing triangles."""
    c = np.asarray(center, dtype=np.float64)
    e = np.asarray(edges, dtype=np.float64)
    n = [max(1, int(round(e[d] / spacing))) for d in range(3)]
    key = {}
    pts = []

    def pid(i, j, k):
        t = (i, j, k)
        if t not in key:
            key[t] = len(pts)
            pts.append(c - 0.5 * e + e * np.array([i / n[0], j / n[1], k / n[2]]))
        return key[t]

    tris = []
    for d in range(3):
        u, w = (d + 1) % 3, (d + 2) % 3
        for side in (0, n[d]):
            for a in range(n[u]):
                for b in range(n[w]):
                    q = []
                    for da, db in ((0, 0), (1, 0), (1, 1), (0, 1)):
                        idx = [0, 0, 0]
                        idx[d], idx[u], idx[w] = side, a + da, b + db
                        q.append(pid(*idx))
                    if side == 0:
                        q = q[::-1]
                    tris += [(q[0], q[1], q[2]), (q[0], q[2], q[3])]
    return np.array(pts), np.array(tris, dtype=np.int32)


def _edge_rest(x, tris):
    p0, p1, p2 = x[tris[:, 0]], x[tris[:, 1]], x[tris[:, 2]]
    return np.stack([np.linalg.norm(p0 - p1, axis=1),
                     np.linalg.norm(p1 - p2, axis=1),
                     np.linalg.norm(p2 - p0, axis=1)], axis=1)


def assemble(name, parts, params, bonds=None, bond_curve=None, domain_scale=10.0, masses=None, domain=None):
    """parts: list of (points, tris, vel (V,3), flag) with flag False/0 free,
    True/1 fixed, 2 a movable rigid body (mass from `masses[part]`, default
    1). Each part with triangles becomes one surface, in order."""
    xs, vs, fx, ts, ss = [], [], [], [], []
    bodies = {}
    off = 0
    for sid, (p, t, v, fixed) in enumerate(parts):
        xs.append(p)
        vs.append(v)
        fx.append(np.full(len(p), int(fixed), dtype=np.uint8))
        if int(fixed) == 2:
            bodies[sid] = dict(mass=float((masses or {}).get(sid, 1.0)),
                               com=np.asarray(p, dtype=np.float64).mean(axis=0),
                               comv=np.asarray(v, dtype=np.float64).mean(axis=0))
        if t is not None and len(t):
            ts.append(t + off)
            ss.append(np.full(len(t), sid, dtype=np.int32))
        off += len(p)
    x = np.concatenate(xs).astype(np.float64)
    v = np.concatenate(vs).astype(np.float64)
    fixed = np.concatenate(fx)
    tris = np.concatenate(ts).astype(np.int32) if ts else np.zeros((0, 3), np.int32)
    tri_surf = np.concatenate(ss).astype(np.int32) if ss else np.zeros(0, np.int32)
    if bonds is None:
        bonds = np.zeros((0, 2), np.int32)
        bond_curve = np.zeros(0, np.int32)
    bonds = np.asarray(bonds, dtype=np.int32).reshape(-1, 2)
    bond_curve = np.asarray(bond_curve, dtype=np.int32)
    tri_rest = _edge_rest(x, tris) if len(tris) else np.zeros((0, 3))
    bond_rest = (np.linalg.norm(x[bonds[:, 0]] - x[bonds[:, 1]], axis=1)
                 if len(bonds) else np.zeros(0))
    if domain is None:
        lo, hi = x.min(axis=0), x.max(axis=0)
        c, half = 0.5 * (lo + hi), 0.5 * (hi - lo) + 1e-3
        domain = np.concatenate([c - domain_scale * half, c + domain_scale * half])
    p = dict(DEFAULTS)
    p.update(params)
    return Scene(name, x, v, fixed, tris, tri_surf, tri_rest.astype(np.float64), bonds,
                 bond_curve, bond_rest.astype(np.float64), np.asarray(domain, dtype=np.float64), p, bodies)


# ------------------------------------------------------------------ workloads

def cloth_on_sphere(n=33, z=0.30, radius=0.25, sub=3, speed=1.0, noise=0.01, dt=1e-3,
                    h=1e-3, mu=0.3, cr=0.0, seed=0, side=1.0):
    rng = np.random.default_rng(seed)
    cp, ct = grid_cloth(n, side, z)
    cv = np.tile(np.array([0.0, 0.0, -speed]), (len(cp), 1))
    cv += rng.uniform(-noise, noise, size=cv.shape)
    sp, st = icosphere(sub, radius)
    return assemble(f"cloth_on_sphere_{n}", [(cp, ct, cv, False),
                                              (sp, st, np.zeros_like(sp), True)],
                    dict(dt=dt, thickness=h, lam=mu, cr=cr))


def folded_cloth(n=129, dt=5e-4, h=5e-4, seed=0, side=1.0, amp=0.05, vscale=2.0):
    rng = np.random.default_rng(seed)
    p, t = grid_cloth(n, side, 0.0)
    a = rng.uniform(0.2, 1.0, 4)
    f = rng.integers(1, 5, 4)
    g = rng.integers(1, 5, 4)
    z = np.zeros(len(p))
    for k in range(4):
        z += a[k] * np.sin(2 * np.pi * (f[k] * p[:, 0] + g[k] * p[:, 1]))
    p[:, 2] = amp * z
    # v = -vscale * grad(phi), phi = sum_k c_k sin(2 pi w_k . x + th_k)
    c = rng.uniform(0.05, 0.15, 4)
    w = rng.uniform(-2.0, 2.0, (4, 3))
    th = rng.uniform(0, 2 * np.pi, 4)
    grad = np.zeros_like(p)
    for k in range(4):
        arg = 2 * np.pi * (p @ w[k]) + th[k]
        grad += (c[k] * np.cos(arg) * 2 * np.pi)[:, None] * w[k][None, :]
    v = -vscale * grad
    return assemble(f"folded_cloth_{n}", [(p, t, v, False)], dict(dt=dt, thickness=h, lam=DEFAULTS["lam"]))


def strings(nstr=64, nseg=512, seglen=2e-3, dt=1e-3, h=1e-3, seed=0, speed=2.0,
            box_lo=(-0.2, -0.2, -0.15), box_hi=(0.2, 0.2, -0.05), z_range=(0.05, 0.45),
            volume_z=(0.0, 0.5)):
    rng = np.random.default_rng(seed)
    pts, bonds, curve = [], [], []
    off = 0
    for s in range(nstr):
        x = np.array([rng.uniform(-0.15, 0.15), rng.uniform(-0.15, 0.15), rng.uniform(*z_range)])
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        sp = [x.copy()]
        for _ in range(nseg):
            # turn by an angle ~ N(0, 0.3) about a random perpendicular axis
            ang = rng.normal(0.0, 0.3)
            r = rng.normal(size=3)
            r -= r.dot(d) * d
            r /= np.linalg.norm(r)
            d = d * math.cos(ang) + r * math.sin(ang)
            d /= np.linalg.norm(d)
            nx = x + seglen * d
            # keep the walk inside the 0.5^3 volume by reflecting
            for k in range(3):
                lo_k, hi_k = (-0.25, 0.25) if k < 2 else volume_z
                if nx[k] < lo_k or nx[k] > hi_k:
                    d[k] = -d[k]
                    nx = x + seglen * d
            x = nx
            sp.append(x.copy())
        sp = np.array(sp)
        pts.append(sp)
        bonds.append(np.stack([np.arange(nseg), np.arange(1, nseg + 1)], axis=1) + off)
        curve.append(np.full(nseg, s, dtype=np.int32))
        off += nseg + 1
    sp = np.concatenate(pts)
    sv = np.tile(np.array([0.0, 0.0, -speed]), (len(sp), 1))
    bp, bt = box_mesh(box_lo, box_hi)
    # surface 0 = box (the only surface); string points come after it
    parts = [(bp, bt, np.zeros_like(bp), True), (sp, None, sv, False)]
    b = np.concatenate(bonds) + len(bp)
    c = np.concatenate(curve)
    return assemble(f"strings_{nstr}x{nseg}", parts, dict(dt=dt, thickness=h, lam=DEFAULTS["lam"]),
                    bonds=b, bond_curve=c)


def cloth_on_obstacle(n, obstacle, radius, speed, dt=1e-3, h=1e-3, seed=0, noise_rel=0.01, gap=None):
    """A cloth above a sphere (top at z = radius) or a 0.4x0.4x0.1 box (top at
    z = 0.05), `gap` above the obstacle's top (default: 0.05 over a sphere,
    0.10 over a box)."""
    rng = np.random.default_rng(seed)
    top = radius if obstacle == "sphere" else 0.05
    if gap is None:
        gap = 0.05 if obstacle == "sphere" else 0.10
    cp, ct = grid_cloth(n, 1.0, top + gap)
    cv = np.tile(np.array([0.0, 0.0, -speed]), (len(cp), 1))
    cv *= 1.0 + rng.uniform(-noise_rel, noise_rel, size=cv.shape)
    if obstacle == "sphere":
        op, ot = icosphere(3, radius)
    else:
        op, ot = box_mesh((-0.2, -0.2, -0.05), (0.2, 0.2, 0.05))
    return assemble(f"cloth_{n}_on_{obstacle}", [(cp, ct, cv, False),
                                                 (op, ot, np.zeros_like(op), True)],
                    dict(dt=dt, thickness=h, lam=DEFAULTS["lam"]))


def batched(nscenes=256, nmin=16, nmax=128, seed=0, dt=1e-3, h=1e-3, approach_steps=(1.0, 4.0)):
    """The batched workload. Each cloth starts above its obstacle by the
    distance it falls in U(approach_steps) steps (drawn from a stream of its
    own, so sizes, obstacles and speeds do not depend on it): every scene is
    in contact from its first few steps on. approach_steps=None places the
    cloths 0.05 above a sphere and 0.10 above a box instead, which the
    slower cloths take up to 200 steps of free fall to cross."""
    rng = np.random.default_rng(seed)
    gap_rng = np.random.default_rng([seed, 0x9a9])
    out = []
    for s in range(nscenes):
        n = int(rng.integers(nmin, nmax + 1))
        obst = "sphere" if rng.random() < 0.5 else "box"
        r = float(rng.uniform(0.1, 0.3))
        speed = float(rng.uniform(0.5, 3.0))
        gap = None
        if approach_steps is not None:
            gap = speed * dt * float(gap_rng.uniform(*approach_steps))
        out.append(cloth_on_obstacle(n, obst, r, speed, dt=dt, h=h, seed=seed * 100003 + s, gap=gap))
    return out


def large(n=1025, sub=5, radius=0.3, speed=10.0, dt=1e-3, h=2e-4, seed=0):
    rng = np.random.default_rng(seed)
    cp, ct = grid_cloth(n, 1.0, radius + 0.02)
    cv = np.tile(np.array([0.0, 0.0, -speed]), (len(cp), 1))
    cv += rng.uniform(-0.01, 0.01, size=cv.shape)
    sp, st = icosphere(sub, radius, (-0.1, 0.0, 0.0))
    bp, bt = box_mesh((0.25, -0.1, -0.1), (0.45, 0.1, 0.1))
    return assemble(f"large_{n}", [(cp, ct, cv, False), (sp, st, np.zeros_like(sp), True),
                                   (bp, bt, np.zeros_like(bp), True)],
                    dict(dt=dt, thickness=h, lam=DEFAULTS["lam"]))


# ------------------------------------------------------ the reference's decks
# in-ball_ball, in-ball_plane, in-box_boundary, in-string_box, in-string_slide
# and in-string_string (cdinit.cpp reads them): spheres (centre, radii,
# velocity), cuboids (centre, half edges, velocity) and strings (end points,
# velocity; cdinit.cpp:145-170 splits a string into bonds of about a quarter
# grid cell) on a 50^3 grid over the deck's domain. MOVABLE_BODY_BOUNDARY
# surfaces become movable rigid bodies of mass 1; FIRST_PHYSICS_WAVE_TYPE
# ones are free cloth. FronTier's surface builders are not available, so
# spheres are icospheres and cuboids are closed grids of about one cell.
# `advance` moves every part along its velocity by that many seconds first,
# so that a short run reaches contact.

_DECKS = {
    "ball_ball": dict(domain=(0, 0, 0, 0.5, 0.5, 0.5), parts=[
        ("sphere", (0.3, 0.3, 0.3), 0.05, (-0.2, -0.2, -0.2), 0),
        ("sphere", (0.2, 0.2, 0.2), 0.05, (0.2, 0.2, 0.2), 0)]),
    "ball_plane": dict(domain=(0, 0, 0.25, 0.5, 0.5, 0.75), parts=[
        ("sphere", (0.25, 0.25, 0.4), 0.05, (0.0, 0.0, 0.2), 2),
        ("cuboid", (0.25, 0.25, 0.47), (0.15, 0.15, 0.01), (0.0, 0.0, -0.2), 0)]),
    "box_boundary": dict(domain=(0, 0, 0, 1.0, 0.5, 0.5), parts=[
        ("cuboid", (0.25, 0.25, 0.21), (0.1, 0.1, 0.2), (0.4, 0.0, -0.4), 2)]),
    "string_box": dict(domain=(0, 0, 0, 0.5, 0.5, 0.5), parts=[
        ("cuboid", (0.25, 0.25, 0.3), (0.15, 0.15, 0.03), (0.0, 0.0, -0.2), 0),
        ("string", (0.25, 0.01, 0.25), (0.25, 0.49, 0.25), (0.0, 0.0, 0.0), 0)]),
    "string_slide": dict(domain=(0, 0, 0, 0.5, 0.5, 0.5), parts=[
        ("cuboid", (0.25, 0.25, 0.13), (0.2, 0.2, 0.02), (0.0, 0.0, 0.0), 2),
        ("string", (0.25, 0.1, 0.3), (0.25, 0.25, 0.155), (0.0, 0.1, -0.1), 0)]),
    "string_string": dict(domain=(0, 0, 0, 0.5, 0.5, 0.5), parts=[
        ("string", (0.25, 0.01, 0.24), (0.25, 0.49, 0.24), (0.0, 0.0, 0.2), 0),
        ("string", (0.01, 0.25, 0.25), (0.49, 0.25, 0.25), (0.0, 0.0, -0.2), 0)]),
}


def deck(name: str, advance: float = 0.0, dt: float = 1e-3, h: float = 1e-3, sub: int = 3, mu: float = 0.0,
         cells: int = 50) -> Scene:
    """One of the reference's decks as a mesh scene (see above)."""
    spec = _DECKS[name]
    dom = np.asarray(spec["domain"], dtype=np.float64)
    cell = float(dom[3] - dom[0]) / cells
    parts, strings = [], []
    for kind, a, b, vel, flag in spec["parts"]:
        vel = np.asarray(vel, dtype=np.float64)
        if kind == "sphere":
            p, t = icosphere(sub, b, center=a)
        elif kind == "cuboid":
            p, t = cuboid_mesh(a, 2.0 * np.asarray(b), cell)
        else:
            e0, e1 = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
            nb = max(1, int(np.linalg.norm(e1 - e0) / (0.25 * cell)))
            p = e0 + np.linspace(0.0, 1.0, nb + 1)[:, None] * (e1 - e0)
            t = None
        p = np.asarray(p, dtype=np.float64) + advance * vel
        v = np.tile(vel, (len(p), 1))
        if t is None:
            strings.append(len(parts))
        parts.append((p, t, v, flag))
    # strings after every surface, as assembleFromInterface lists them
    order = [i for i in range(len(parts)) if i not in strings] + strings
    parts = [parts[i] for i in order]
    bonds, curve, off = [], [], 0
    for ci, (p, t, v, flag) in enumerate(parts):
        if t is None:
            n = len(p) - 1
            bonds.append(np.stack([np.arange(n), np.arange(1, n + 1)], axis=1) + off)
            curve.append(np.full(n, ci, dtype=np.int32))
        off += len(p)
    b = np.concatenate(bonds) if bonds else None
    c = np.concatenate(curve) if curve else None
    return assemble(f"deck_{name}", parts, dict(dt=dt, thickness=h, lam=mu), bonds=b, bond_curve=c, domain=dom)


def workload(name: str, seed: int = 0):
    """The five measured workloads by name."""
    if name == "cloth_on_sphere":
        return [cloth_on_sphere(seed=seed)]
    if name == "folded_cloth":
        return [folded_cloth(seed=seed)]
    if name == "strings":
        return [strings(seed=seed)]
    if name == "batched":
        return batched(seed=seed)
    if name == "large":
        return [large(seed=seed)]
    raise KeyError(name)


def candidate(scene: Scene, x_old: np.ndarray, vel: np.ndarray) -> np.ndarray:
    """The host loop's candidate positions x_old + dt*vel (test.cpp:238)."""
    return x_old + scene.params["dt"] * vel
