"""The strain schedule builder, on the CPU.

Strain limiting in the reference is one sequential sweep over the element
edges (dcollid.cpp:586-596). The runtime sweeps it level by level on the GPU,
with each point's velocity held in a shared-memory slot for its live interval
(collision_gb300/csrc/cc_strain_plan.cpp). That file is compiled here with g++
and its schedule is checked against the properties the sweep relies on.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from collision_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = "/usr/local/cuda/include"
AHEAD = 8  # kStrainAhead: copy-ins run this many levels before a point's first edge


def compile_plan(gxx, plan_cpp, so):
    """Builds the shim around a copy of the schedule builder into so."""
    src = os.path.join(ROOT, "collision_gb300", "csrc")
    subprocess.run([gxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I", src, "-I", CUDA_INC,
                    os.path.join(ROOT, "tests", "strain_plan_shim.cpp"), plan_cpp, "-o", so], check=True)
    return load_plan(so)


@pytest.fixture(scope="module")
def plan(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx or not os.path.isdir(CUDA_INC):
        pytest.skip("needs g++ and the CUDA headers")
    so = str(tmp_path_factory.mktemp("strain_plan") / "libstrain_plan.so")
    return compile_plan(gxx, os.path.join(ROOT, "collision_gb300", "csrc", "cc_strain_plan.cpp"), so)


def load_plan(so):
    """The schedule of one scene's edges, through the shim in library so."""
    lib = C.CDLL(so)
    ip = C.POINTER(C.c_int)
    lib.strain_plan.restype = C.c_int
    lib.strain_plan.argtypes = [ip, ip, C.c_int, C.c_int, C.c_int, ip, ip, C.c_int, ip, ip, C.c_int, ip]

    def run(edges, v0, nv):
        e = np.ascontiguousarray(edges, np.int32)
        m = len(e)
        p0, p1 = np.ascontiguousarray(e[:, 0]), np.ascontiguousarray(e[:, 1])
        out = np.empty((m, 4), np.int32)
        hdr = np.empty((2 * m + 2, 4), np.int32)
        load = np.empty((nv, 2), np.int32)
        wb = np.empty((nv, 2), np.int32)
        info = np.empty(9, np.int32)
        ptr = lambda a: a.ctypes.data_as(ip)  # noqa: E731
        rc = lib.strain_plan(ptr(p0), ptr(p1), m, v0, nv, ptr(out), ptr(hdr), len(hdr), ptr(load), ptr(wb), nv,
                             ptr(info))
        assert rc == 0
        levels, slots, wf0, wf1, cap_e, cap_l, cap_w, nload, nwb = (int(v) for v in info)
        return dict(edges=out, hdr=hdr[:2 * levels], load=load[:nload], wb=wb[:nwb], levels=levels, slots=slots,
                    wb_final=(wf0, wf1), caps=(cap_e, cap_l, cap_w))
    return run


def _reference_edges(sc, v0):
    """The sweep's edges in the reference's order: elements in order, a
    triangle's sides p0p1, p1p2, p2p0, then the bonds."""
    t = np.asarray(sc.tris, np.int64)
    tri_edges = np.stack([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]], axis=1).reshape(-1, 2)
    edges = np.concatenate([tri_edges, np.asarray(sc.bonds, np.int64).reshape(-1, 2)])
    return edges + v0


@pytest.mark.parametrize("make", [
    lambda: scenes.cloth_on_sphere(n=12, sub=1, seed=1),
    lambda: scenes.folded_cloth(n=33, seed=1),
    lambda: scenes.strings(nstr=6, nseg=64, seed=4),
], ids=["cloth12", "folded33", "strings"])
def test_strain_schedule_properties(plan, make):
    sc = make()
    v0 = 1000  # batch point ids start at the scene's first point
    edges = _reference_edges(sc, v0)
    r = plan(edges, v0, sc.nv)
    out, hdr, levels = r["edges"], r["hdr"], r["levels"]
    ebase = hdr[0, 0]
    assert ebase == 0 and hdr[2 * levels - 2, 1] == len(edges)

    # the levels partition the edges, each in the input order within a level
    level_of = np.empty(len(edges), np.int64)
    pos = {}
    for i, (a, b) in enumerate(map(tuple, edges)):
        pos.setdefault((a, b), []).append(i)
    seen = {}
    for l in range(levels):
        lo, hi = hdr[2 * l, 0], hdr[2 * l, 1]
        lev = out[lo:hi]
        pts = lev[:, :2].ravel()
        assert len(np.unique(pts)) == len(pts), f"level {l}: two edges share a point"
        prev = -1
        for a, b in map(tuple, lev[:, :2]):
            k = seen.get((a, b), 0)
            i = pos[(a, b)][k]
            seen[(a, b)] = k + 1
            level_of[i] = l
            assert i > prev, "edges of one level keep the input order"
            prev = i
    assert sum(seen.values()) == len(edges)

    # two edges at one point keep the reference's order across levels
    last = {}
    for i, (a, b) in enumerate(map(tuple, edges)):
        for p in (a, b):
            if p in last:
                assert level_of[last[p]] < level_of[i], "a later edge at a point swept first"
            last[p] = i

    # each point's slot, first and last level, copy-in and write-back
    first_l, last_l, slot = {}, {}, {}
    for l in range(levels):
        for a, b, s0, s1 in out[hdr[2 * l, 0]:hdr[2 * l, 1]]:
            for p, s in ((a, s0), (b, s1)):
                first_l.setdefault(p, l)
                last_l[p] = l
                assert slot.setdefault(p, s) == s, "a point changes slot"
    load_level = {}
    for l in range(levels):
        for p, s in r["load"][hdr[2 * l, 2] - hdr[0, 2]:hdr[2 * l, 3] - hdr[0, 2]]:
            assert p not in load_level and slot[p] == s
            load_level[p] = l
    wb_level = {}
    wb0 = hdr[1, 0]
    for l in range(levels):
        for p, s in r["wb"][hdr[2 * l + 1, 0] - wb0:hdr[2 * l + 1, 1] - wb0]:
            assert p not in wb_level and slot[p] == s
            wb_level[p] = l
    for p, s in r["wb"][r["wb_final"][0] - wb0:r["wb_final"][1] - wb0]:
        assert p not in wb_level and slot[p] == s
        wb_level[p] = levels
    assert set(load_level) == set(first_l) == set(wb_level)
    for p in first_l:
        assert load_level[p] == max(0, first_l[p] - AHEAD)
        assert wb_level[p] == last_l[p] + 1

    # points sharing a slot have disjoint live intervals (copy-in .. write-back)
    by_slot = {}
    for p, s in slot.items():
        by_slot.setdefault(s, []).append((load_level[p], wb_level[p]))
    assert len(by_slot) == r["slots"]
    for s, iv in by_slot.items():
        iv.sort()
        for (c0, w0), (c1, w1) in zip(iv, iv[1:]):
            assert c1 > w0, f"slot {s}: a copy-in at level {c1} before the write-back at level {w0}"

    # the per-level maxima the sweep sizes its block with
    assert r["caps"][0] == max(hdr[2 * l, 1] - hdr[2 * l, 0] for l in range(levels))
    assert r["caps"][1] == max(hdr[2 * l, 3] - hdr[2 * l, 2] for l in range(levels))
    assert r["caps"][2] == max(hdr[2 * l + 1, 1] - hdr[2 * l + 1, 0] for l in range(levels))
