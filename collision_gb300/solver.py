"""CollisionSolver3d: the reference's solver surface over the GPU library.

Mirrors antdvid/Collision's CollisionSolver3d (collid.h:128-244): the
parameter setters (there class statics, collid.h:180-193; here per solver),
setDomainBoundary, resolveCollision and hasCollision. assembleFromMesh takes
triangle / bond lists and replaces assembleFromInterface (collid.h:242),
whose FronTier interface is not part of this library.

Positions and velocities are numpy arrays of shape (n_points, 3) float64 on
the host (resolveCollision: copies inside the call) or torch CUDA tensors
(resolveCollisionDevice: no copies).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .scenes import DEFAULTS, PARAM_NAMES


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


class CollisionSolver3d:
    def __init__(self, device: int = 0):
        self._lib = _lib.load()
        h = C.c_void_p()
        st = self._lib.cc_create(int(device), C.byref(h))
        if st != 0:
            raise _lib.CCError(st, f"cc_create(device={device}) failed")
        self._h = h
        self._params = dict(DEFAULTS)
        self._has_collision = False
        self._nv = 0
        self._ne = 0
        self._push_params()

    # ------------------------------------------------------------ lifetime
    def close(self):
        if getattr(self, "_h", None):
            self._lib.cc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != 0:
            buf = C.create_string_buffer(512)
            self._lib.cc_last_error(self._h, buf, 512)
            raise _lib.CCError(st, buf.value.decode(errors="replace"))

    # --------------------------------------------------------- parameters
    def _push_params(self):
        p = _lib.cc_params(*[float(self._params[k]) for k in PARAM_NAMES])
        self._check(self._lib.cc_set_params(self._h, C.byref(p)))

    def _set(self, k, v):
        self._params[k] = float(v)
        self._push_params()

    def setTimeStepSize(self, dt): self._set("dt", dt)
    def getTimeStepSize(self): return self._params["dt"]
    def setFabricThickness(self, h): self._set("thickness", h)
    def getFabricThickness(self): return self._params["thickness"]
    def setRoundingTolerance(self, eps): self._set("eps", eps)
    def getRoundingTolerance(self): return self._params["eps"]
    def setSpringConstant(self, k): self._set("k", k)
    def getSpringConstant(self): return self._params["k"]
    def setPointMass(self, m): self._set("m", m)
    def getPointMass(self): return self._params["m"]
    def setFrictionConstant(self, lam): self._set("lam", lam)
    def getFrictionConstant(self): return self._params["lam"]
    def setRestitutionCoef(self, cr): self._set("cr", cr)
    def getRestitutionCoef(self): return self._params["cr"]

    def setParams(self, params: dict):
        self._params.update({k: float(v) for k, v in params.items() if k in PARAM_NAMES})
        self._push_params()

    def setDomainBoundary(self, L, U):
        lo = _c(L, np.float64)
        hi = _c(U, np.float64)
        self._check(self._lib.cc_set_domain_boundary(self._h, lo.ctypes.data, hi.ctypes.data))

    # ------------------------------------------------------------- mesh
    def assembleFromMesh(self, n_points, tris=None, tri_surface=None, tri_rest=None, bonds=None,
                         bond_rest=None, fixed=None):
        tris = _c(tris if tris is not None else np.zeros((0, 3)), np.int32).reshape(-1, 3)
        nt = tris.shape[0]
        tri_surface = _c(tri_surface if tri_surface is not None else np.zeros(nt), np.int32)
        tri_rest = _c(tri_rest if tri_rest is not None else np.zeros((nt, 3)), np.float64).reshape(-1, 3)
        bonds = _c(bonds if bonds is not None else np.zeros((0, 2)), np.int32).reshape(-1, 2)
        nb = bonds.shape[0]
        bond_rest = _c(bond_rest if bond_rest is not None else np.zeros(nb), np.float64)
        fixed = _c(fixed if fixed is not None else np.zeros(n_points), np.uint8)
        self._keep = (tris, tri_surface, tri_rest, bonds, bond_rest, fixed)
        m = _lib.cc_mesh(int(n_points), nt, tris.ctypes.data, tri_surface.ctypes.data, tri_rest.ctypes.data,
                         nb, bonds.ctypes.data, bond_rest.ctypes.data, fixed.ctypes.data)
        self._check(self._lib.cc_assemble(self._h, C.byref(m)))
        self._nv = int(n_points)
        self._ne = nt + nb

    def assembleFromScene(self, scene):
        """Mesh, parameters and domain of a collision_gb300.scenes.Scene."""
        self.assembleFromMesh(scene.nv, scene.tris, scene.tri_surf, scene.tri_rest, scene.bonds,
                              scene.bond_rest, scene.fixed)
        self.setParams(scene.params)
        self.setDomainBoundary(scene.domain[:3], scene.domain[3:])
        for sid, b in sorted(scene.bodies.items()):
            self.setBody(sid, b["mass"], b["com"], b["comv"])

    # ------------------------------------------------------------ batches
    def assembleBatch(self, meshes):
        """Several independent scenes in one solver. `meshes` holds dicts with
        the keyword arguments of assembleFromMesh, or Scene objects (whose
        parameters and domain boxes are applied per scene). Points and
        elements are numbered scene by scene (sceneOffsets)."""
        from .scenes import Scene
        keep, cms, scene_objs = [], [], []
        for m in meshes:
            if isinstance(m, Scene):
                scene_objs.append(m)
                m = dict(n_points=m.nv, tris=m.tris, tri_surface=m.tri_surf, tri_rest=m.tri_rest, bonds=m.bonds,
                         bond_rest=m.bond_rest, fixed=m.fixed)
            else:
                scene_objs.append(None)
            n_points = int(m["n_points"])
            tris = _c(m.get("tris") if m.get("tris") is not None else np.zeros((0, 3)), np.int32).reshape(-1, 3)
            nt = tris.shape[0]
            ts = m.get("tri_surface")
            ts = _c(ts if ts is not None else np.zeros(nt), np.int32)
            tr = m.get("tri_rest")
            tr = _c(tr if tr is not None else np.zeros((nt, 3)), np.float64).reshape(-1, 3)
            bonds = _c(m.get("bonds") if m.get("bonds") is not None else np.zeros((0, 2)), np.int32).reshape(-1, 2)
            nb = bonds.shape[0]
            br = m.get("bond_rest")
            br = _c(br if br is not None else np.zeros(nb), np.float64)
            fx = m.get("fixed")
            fx = _c(fx if fx is not None else np.zeros(n_points), np.uint8)
            keep.append((tris, ts, tr, bonds, br, fx))
            cms.append(_lib.cc_mesh(n_points, nt, tris.ctypes.data, ts.ctypes.data, tr.ctypes.data, nb,
                                    bonds.ctypes.data, br.ctypes.data, fx.ctypes.data))
        arr = (_lib.cc_mesh * len(cms))(*cms)
        self._check(self._lib.cc_assemble_batch(self._h, arr, len(cms)))
        self._keep = keep
        off_v, off_e = self.sceneOffsets()
        self._nv = int(off_v[-1])
        self._ne = int(off_e[-1])
        for i, sc in enumerate(scene_objs):
            if sc is not None:
                self.setSceneParams(i, sc.params)
                self.setSceneDomainBoundary(i, sc.domain[:3], sc.domain[3:])
                for sid, b in sorted(sc.bodies.items()):
                    self.setBody(sid, b["mass"], b["com"], b["comv"], scene=i)

    def numScenes(self) -> int:
        return int(self._lib.cc_num_scenes(self._h))

    def sceneOffsets(self):
        """(point offsets, element offsets), n_scenes + 1 entries each."""
        n = self.numScenes()
        pv = np.zeros(n + 1, dtype=np.int32)
        pe = np.zeros(n + 1, dtype=np.int32)
        self._check(self._lib.cc_get_scene_offsets(self._h, pv.ctypes.data_as(C.POINTER(C.c_int)),
                                                   pe.ctypes.data_as(C.POINTER(C.c_int))))
        return pv, pe

    def setSceneParams(self, scene: int, params: dict):
        vals = dict(self._params)
        vals.update({k: float(v) for k, v in params.items() if k in PARAM_NAMES})
        p = _lib.cc_params(*[float(vals[k]) for k in PARAM_NAMES])
        self._check(self._lib.cc_set_scene_params(self._h, int(scene), C.byref(p)))

    def setSceneDomainBoundary(self, scene: int, L, U):
        lo = _c(L, np.float64)
        hi = _c(U, np.float64)
        self._check(self._lib.cc_set_scene_domain_boundary(self._h, int(scene), lo.ctypes.data, hi.ctypes.data))

    TUNE_SPLIT_NARROW, TUNE_TRAVERSE_BLOCK, TUNE_NARROW_BLOCK, TUNE_STRAIN_BLOCK, TUNE_TAIL_GRAPH = 0, 1, 2, 3, 4
    TUNE_COMBINED_BROAD, TUNE_STRAIN_WARP, TUNE_PACKET_TRAVERSE, TUNE_STRAIN_ROLES, TUNE_TAIL_OVERLAP = 5, 6, 7, 8, 9
    TUNE_ROPE_TRAVERSE, TUNE_SUBSET_REFIT, TUNE_TRAVERSE_REFILL, TUNE_STACK_DEPTH, TUNE_PAIR_CAPACITY = 10, 11, 12, 13, 14
    TUNE_DEVICE_LOOP, TUNE_PRUNE, TUNE_HOST_TREE, TUNE_SMALL_SORT, TUNE_PRUNED_WARP = 15, 16, 17, 18, 19
    TUNE_ROBUST_ROOTS, TUNE_ZONE_CTA_MIN, TUNE_REPLAY_CTA_MIN, TUNE_REFIT_UP, TUNE_ZONE_FEW = 20, 21, 22, 23, 24
    TUNE_SUBTEST_MERGE = 25

    def setTuning(self, knob: int, value: int):
        """Launch shapes and the two-stage narrow phase; none changes results."""
        self._check(self._lib.cc_set_tuning(self._h, int(knob), int(value)))

    def getTuning(self, knob: int) -> int:
        return int(self._lib.cc_get_tuning(self._h, int(knob)))

    def autotune(self) -> dict:
        """Pick launch shapes on the current state (after a resolve call);
        returns the chosen settings and the best timed pass in ms."""
        ms = C.c_double(0.0)
        self._check(self._lib.cc_autotune(self._h, C.byref(ms)))
        return {"packet_traverse": self.getTuning(self.TUNE_PACKET_TRAVERSE),
                "rope_traverse": self.getTuning(self.TUNE_ROPE_TRAVERSE),
                "traverse_refill": self.getTuning(self.TUNE_TRAVERSE_REFILL),
                "stack_depth": self.getTuning(self.TUNE_STACK_DEPTH),
                "pair_capacity": self.getTuning(self.TUNE_PAIR_CAPACITY),
                "traverse_block": self.getTuning(self.TUNE_TRAVERSE_BLOCK),
                "split_narrow": self.getTuning(self.TUNE_SPLIT_NARROW),
                "narrow_block": self.getTuning(self.TUNE_NARROW_BLOCK), "pass_ms": ms.value}

    def setVtkDump(self, directory):
        """Write a .vtp of every detection pass into `directory` (None: off)."""
        d = None if directory is None else str(directory).encode()
        self._check(self._lib.cc_set_vtk_dump(self._h, d))

    def setBody(self, surface: int, mass: float, com, comv, scene: int = 0):
        """Mass, centre of mass and centre-of-mass velocity (the HYPER_SURF
        data) of the movable rigid body formed by surface `surface`."""
        com = np.ascontiguousarray(com, dtype=np.float64)
        comv = np.ascontiguousarray(comv, dtype=np.float64)
        dp = C.POINTER(C.c_double)
        self._check(self._lib.cc_set_body(self._h, int(scene), int(surface), float(mass), com.ctypes.data_as(dp),
                                          comv.ctypes.data_as(dp)))

    def body(self, surface: int, scene: int = 0):
        """(centre of mass, centre-of-mass velocity) of a movable body after
        the last step (updateFinalForRG)."""
        com, comv = np.zeros(3), np.zeros(3)
        dp = C.POINTER(C.c_double)
        self._check(self._lib.cc_get_body(self._h, int(scene), int(surface), com.ctypes.data_as(dp),
                                          comv.ctypes.data_as(dp)))
        return com, comv

    def setZoneCap(self, cap: int):
        """Impact-zone passes per scene and step before the loop is stopped."""
        self._check(self._lib.cc_set_zone_cap(self._h, int(cap)))

    def setSceneEnabled(self, scene: int, on: bool):
        self._check(self._lib.cc_set_scene_enabled(self._h, int(scene), int(bool(on))))

    def sceneStatus(self) -> np.ndarray:
        """Status of every scene in the last resolve call (0, or 4 = CC_ITER_CAP)."""
        out = np.zeros(max(self.numScenes(), 1), dtype=np.int32)
        self._check(self._lib.cc_get_scene_status(self._h, out.ctypes.data_as(C.POINTER(C.c_int))))
        return out[:self.numScenes()]

    def setHostThreads(self, n: int):
        self._check(self._lib.cc_set_host_threads(self._h, int(n)))

    def resolveCollisionBatch(self, x_old, x_cand, vel, has_collsn):
        """resolveCollision() on every scene (host arrays over all scenes'
        points). Returns (x_new, vel, has_collsn, has_collision per scene)."""
        x_old = _c(x_old, np.float64)
        x_cand = _c(x_cand, np.float64)
        vel = np.array(vel, dtype=np.float64, copy=True, order="C")
        hc = np.array(has_collsn, dtype=np.uint8, copy=True, order="C")
        x_out = np.empty_like(x_old)
        hcol = np.zeros(max(self.numScenes(), 1), dtype=np.int32)
        st = self._lib.cc_resolve_batch(self._h, x_old.ctypes.data, x_cand.ctypes.data, vel.ctypes.data,
                                        hc.ctypes.data, x_out.ctypes.data, hcol.ctypes.data_as(C.POINTER(C.c_int)))
        if st != self.ITER_CAP:  # scenes that reached the zone cap: see sceneStatus()
            self._check(st)
        self._has_collision = bool(hcol.any())
        return x_out, vel, hc, hcol.astype(bool)

    def resolveCollisionBatchDevice(self, x_old, x_cand, vel, has_collsn, x_out):
        """resolveCollision() on every scene, device tensors as in
        resolveCollisionDevice. Returns has_collision per scene."""
        hcol = np.zeros(max(self.numScenes(), 1), dtype=np.int32)
        st = self._lib.cc_resolve_batch_device(self._h, x_old.data_ptr(), x_cand.data_ptr(), vel.data_ptr(),
                                               has_collsn.data_ptr(), x_out.data_ptr(),
                                               hcol.ctypes.data_as(C.POINTER(C.c_int)))
        if st != self.ITER_CAP:
            self._check(st)
        self._has_collision = bool(hcol.any())
        return hcol.astype(bool)

    def checkCCD(self, x_old, x_new):
        """Exact FP64 CCD re-check of a finished step on device tensors:
        (element pairs that still collide, per-scene counts)."""
        hits = C.c_longlong(0)
        per = np.zeros(max(self.numScenes(), 1), dtype=np.int32)
        self._check(self._lib.cc_check_ccd(self._h, x_old.data_ptr(), x_new.data_ptr(), C.byref(hits),
                                           per.ctypes.data_as(C.POINTER(C.c_int))))
        return int(hits.value), per

    def scenePassKinds(self, scene: int) -> np.ndarray:
        n = self._lib.cc_get_scene_pass_kinds(self._h, int(scene), None, 0)
        out = np.zeros(max(n, 0), dtype=np.int32)
        if n > 0:
            self._lib.cc_get_scene_pass_kinds(self._h, int(scene), out.ctypes.data_as(C.POINTER(C.c_int)), n)
        return out

    # -------------------------------------------------------------- step
    def resolveCollision(self, x_old, x_cand, vel, has_collsn):
        """One resolveCollision() on host arrays. Returns (x_new, vel, has_collsn)."""
        x_old = _c(x_old, np.float64)
        x_cand = _c(x_cand, np.float64)
        vel = np.array(vel, dtype=np.float64, copy=True, order="C")
        hc = np.array(has_collsn, dtype=np.uint8, copy=True, order="C")
        x_out = np.empty_like(x_old)
        hcol = C.c_int(0)
        self._check(self._lib.cc_resolve(self._h, x_old.ctypes.data, x_cand.ctypes.data, vel.ctypes.data,
                                         hc.ctypes.data, x_out.ctypes.data, C.byref(hcol)))
        self._has_collision = bool(hcol.value)
        return x_out, vel, hc

    def resolveCollisionDevice(self, x_old, x_cand, vel, has_collsn, x_out):
        """One resolveCollision() on device tensors (torch, on this solver's
        device, contiguous float64 / uint8). vel and has_collsn are updated in
        place; x_out receives the final positions."""
        hcol = C.c_int(0)
        self._check(self._lib.cc_resolve_device(self._h, x_old.data_ptr(), x_cand.data_ptr(), vel.data_ptr(),
                                                has_collsn.data_ptr(), x_out.data_ptr(), C.byref(hcol)))
        self._has_collision = bool(hcol.value)

    def setStream(self, stream_handle: int | None):
        """Run on a caller's CUDA stream (e.g. torch.cuda.current_stream().cuda_stream)."""
        self._check(self._lib.cc_set_stream(self._h, stream_handle))

    PLAIN_FP64, MIXED = 0, 1
    ITER_CAP = 4

    def setMode(self, mode: int):
        """0: plain FP64; 1: FP32 filters in front of the same FP64 tests."""
        self._check(self._lib.cc_set_mode(self._h, int(mode)))

    def setStrainWindow(self, on: bool):
        """Shared-memory window for the strain sweep (default) or global memory."""
        self._check(self._lib.cc_set_strain_window(self._h, int(bool(on))))

    def setProfiling(self, on):
        """Stage timing: True/1 outside the device loop's graph, 2 also per
        stage inside it, False/0 off."""
        self._check(self._lib.cc_set_profiling(self._h, int(on)))

    def profile(self) -> dict:
        ms = (C.c_double * 32)()
        calls = (C.c_longlong * 32)()
        n = self._lib.cc_get_profile(self._h, ms, calls, 32)
        return {self._lib.cc_profile_stage_name(i).decode(): (ms[i], calls[i]) for i in range(n)}

    def hasCollision(self) -> bool:
        return self._has_collision

    # ------------------------------------------------------- inspection
    COUNTER_NAMES = ("passes", "ccd_passes", "zone_passes", "candidate_pairs", "visits", "hit_pairs",
                     "contacts", "strain_passes", "tree_builds", "kernel_launches", "strain_averaged",
                     "strain_exact", "fp64_subtests", "moving_visits", "strain_bytes", "cr_roots", "broad_leaves",
                     "broad_pairs", "path_bytes", "timed_traverse_leaves", "timed_traverse_pairs", "loop_passes",
                     "tree_build_us", "pruned_queries", "zone_unions")

    def counters(self) -> dict:
        n_all = len(self.COUNTER_NAMES)
        out = (C.c_longlong * n_all)()
        n = self._lib.cc_get_counters(self._h, out, n_all)
        return dict(zip(self.COUNTER_NAMES[:n], list(out)[:n]))

    def setRecording(self, on: bool):
        self._check(self._lib.cc_set_recording(self._h, int(bool(on))))

    def visits(self) -> np.ndarray:
        """(n, 13) int32: pass, kind, a, b, status, dcount[6], rank_b, rank_a."""
        n = self._lib.cc_get_visits(self._h, None, 0)
        out = np.zeros((max(n, 0), 13), dtype=np.int32)
        if n > 0:
            self._lib.cc_get_visits(self._h, out.ctypes.data_as(C.POINTER(C.c_int)), n)
        return out

    def passKinds(self) -> np.ndarray:
        n = self._lib.cc_get_pass_kinds(self._h, None, 0)
        out = np.zeros(max(n, 0), dtype=np.int32)
        if n > 0:
            self._lib.cc_get_pass_kinds(self._h, out.ctypes.data_as(C.POINTER(C.c_int)), n)
        return out

    def zoneRoots(self) -> np.ndarray:
        out = np.zeros(self._nv, dtype=np.int32)
        self._check(self._lib.cc_get_zone_roots(self._h, out.ctypes.data_as(C.POINTER(C.c_int))))
        return out

    def leafRanks(self, which: int):
        out = np.zeros(self._ne, dtype=np.int32)
        st = self._lib.cc_get_leaf_ranks(self._h, int(which), out.ctypes.data_as(C.POINTER(C.c_int)))
        return out if st == 0 else None

    def treeVolume(self, scene: int = 0) -> float:
        """Root volume of the scene's last built tree (both trees share it)."""
        v = C.c_double(0.0)
        self._check(self._lib.cc_get_tree_volume(self._h, int(scene), C.byref(v)))
        return v.value

    def candidatePairs(self, moving: bool, brute_force: bool = False) -> np.ndarray:
        n = self._lib.cc_debug_candidate_pairs(self._h, int(moving), int(brute_force), None, 0)
        if n < 0:
            self._check(2)
        out = np.zeros((n, 2), dtype=np.int32)
        if n:
            self._lib.cc_debug_candidate_pairs(self._h, int(moving), int(brute_force),
                                               out.ctypes.data_as(C.POINTER(C.c_int)), n)
        return out


def ordered_visits(v: np.ndarray) -> np.ndarray:
    """GPU visit records in the reference's visiting order: by pass, then
    query-leaf rank, then found-leaf rank; returns the 11-column oracle form."""
    if len(v) == 0:
        return np.zeros((0, 11), dtype=np.int32)
    idx = np.lexsort((v[:, 12], v[:, 11], v[:, 0]))
    return v[idx, :11]
