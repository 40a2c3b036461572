"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference's own CollisionSolver3d (AABB.cpp, dcollid.cpp,
dcollid3d.cpp compiled unmodified against the stub headers by
oracle/Makefile.ref) through the reference host loop on small seeded scenes,
and stores per step:
  inputs   x_old, x_cand, vel, has_collsn (left out for the cases in
           cases.CHAINED, whose inputs are the previous step's outputs)
  outputs  x, vel, has_collsn, has_collision, impact-zone labels, and the
           centre of mass and its velocity of every movable body
  trace    pass kinds; every narrow-phase call that hit (pass, kind, a, b,
           status, collsn_num increments); the count and SHA-256 of the full
           visit record (every call, in order, with orientation)

Needs the reference sources (--ref or CC_REFERENCE; default: a directory
named reference beside the repository) and g++. The
fixtures it writes are self-contained: tests read only the .npz files.

    python tests/golden/make_golden.py [--ref /path/to/reference]
"""
from __future__ import annotations

import argparse
import hashlib
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from collision_gb300 import scenes  # noqa: E402
from tests.golden.cases import CASES, CHAINED  # noqa: E402


def pair_hash(pairs: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(pairs, dtype="<i4").tobytes()).hexdigest()


def zone_labels(zone_root):
    zr = np.asarray(zone_root)
    lab = np.arange(len(zr))
    mins = {}
    for i, r in enumerate(zr):
        mins[r] = min(mins.get(r, i), i)
    return np.array([mins[r] for r in zr], dtype=np.int32)


def run_case(name, make, nsteps):
    from oracle.refpy import RefSolver
    sc = make()
    ref = RefSolver(sc, record=True)
    x = sc.x.copy()
    v = sc.v.copy()
    hc = np.zeros(sc.nv, np.uint8)
    rec = {k: [] for k in ("x_old", "x_cand", "vel_in", "hc_in", "x", "vel", "hc", "has_collision",
                           "zones", "npairs", "pair_sha", "body_com", "body_comv")}
    body_ids = sorted(sc.bodies)
    hits, kinds = [], []
    for step in range(nsteps):
        xc = scenes.candidate(sc, x, v)
        out = ref.step(x, xc, v, hc)
        if out["rc"] != 0:
            raise RuntimeError(f"{name}: reference exited with {out['rc']} at step {step}")
        p = ref.pairs()
        rec["x_old"].append(x); rec["x_cand"].append(xc); rec["vel_in"].append(v); rec["hc_in"].append(hc)
        rec["x"].append(out["x"]); rec["vel"].append(out["v"]); rec["hc"].append(out["has_collsn"])
        rec["has_collision"].append(out["has_collision"])
        rec["zones"].append(zone_labels(out["zone_root"]))
        rec["npairs"].append(len(p))
        rec["pair_sha"].append(pair_hash(p))
        h = p[p[:, 4] != 0]
        hits.append(np.concatenate([np.full((len(h), 1), step, np.int32), h], axis=1))
        k = ref.passes()
        kinds.append(np.stack([np.full(len(k), step, np.int32), k], axis=1))
        bodies = [ref.body(b) for b in body_ids]
        rec["body_com"].append(np.array([b[0] for b in bodies]).reshape(-1, 3))
        rec["body_comv"].append(np.array([b[1] for b in bodies]).reshape(-1, 3))
        x, v, hc = out["x"], out["v"], out["has_collsn"]
    ref.close()
    if name in CHAINED:
        for k in ("x_old", "x_cand", "vel_in", "hc_in"):
            del rec[k]
    arrs = {k: np.array(val) for k, val in rec.items()}
    arrs["hits"] = np.concatenate(hits) if hits else np.zeros((0, 12), np.int32)
    arrs["pass_kinds"] = np.concatenate(kinds)
    for f in ("tris", "tri_surf", "tri_rest", "bonds", "bond_curve", "bond_rest", "fixed", "domain"):
        arrs["scene_" + f] = getattr(sc, f)
    arrs["scene_params"] = sc.param_vec()
    arrs["scene_body_surf"] = np.array(body_ids, dtype=np.int32)
    arrs["scene_body_mass"] = np.array([sc.bodies[b]["mass"] for b in body_ids], dtype=np.float64)
    arrs["scene_body_com"] = np.array([sc.bodies[b]["com"] for b in body_ids], dtype=np.float64).reshape(-1, 3)
    arrs["scene_body_comv"] = np.array([sc.bodies[b]["comv"] for b in body_ids], dtype=np.float64).reshape(-1, 3)
    arrs["scene_x"] = sc.x
    arrs["scene_v"] = sc.v
    return arrs


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("CC_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference")))
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    subprocess.check_call(["make", "-s", "-f", os.path.join(ROOT, "oracle", "Makefile.ref"),
                           f"REF={args.ref}", "-j4"])
    for name, (make, nsteps) in CASES.items():
        if args.only and name != args.only:
            continue
        arrs = run_case(name, make, nsteps)
        out = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(out, **arrs)
        print(f"{name}: {nsteps} steps, {int(sum(arrs['npairs']))} visits, "
              f"{len(arrs['hits'])} hits -> {os.path.relpath(out, ROOT)} "
              f"({os.path.getsize(out) // 1024} KB)")


if __name__ == "__main__":
    main()
