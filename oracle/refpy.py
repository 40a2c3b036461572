"""ctypes binding to oracle/_ref/libccref.so (the reference's own solver sources
compiled against the stub headers, see oracle/Makefile.ref).

TEST INFRASTRUCTURE ONLY: used to pin the C restatement (oracle/cc_oracle.c)
and to generate tests/golden/. It exists only where the reference sources do
(this is never built on, or shipped to, the GPU host).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libccref.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_up = C.POINTER(C.c_ubyte)


def _ptr(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def available() -> bool:
    return os.path.exists(LIB_PATH)


def load():
    lib = C.CDLL(LIB_PATH)
    lib.ref_create.restype = C.c_void_p
    lib.ref_create.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, C.c_int, _ip, _ip, _dp, _up]
    lib.ref_destroy.argtypes = [C.c_void_p]
    lib.ref_set_recording.argtypes = [C.c_void_p, C.c_int, C.c_int]
    lib.ref_step.restype = C.c_int
    lib.ref_step.argtypes = [C.c_void_p, _dp, _dp, _dp, _up, _dp, _dp, C.c_int, _dp, _dp, _ip, _ip]
    lib.ref_num_passes.restype = C.c_int
    lib.ref_num_passes.argtypes = [C.c_void_p]
    lib.ref_pass_kinds.argtypes = [C.c_void_p, _ip]
    lib.ref_num_pairs.restype = C.c_int
    lib.ref_num_pairs.argtypes = [C.c_void_p]
    lib.ref_pairs.argtypes = [C.c_void_p, _ip]
    lib.ref_num_vel_snaps.restype = C.c_int
    lib.ref_num_vel_snaps.argtypes = [C.c_void_p]
    lib.ref_vel_snaps.argtypes = [C.c_void_p, _dp]
    lib.ref_set_body.restype = C.c_int
    lib.ref_set_body.argtypes = [C.c_void_p, C.c_int, C.c_double, _dp, _dp]
    lib.ref_get_body.restype = C.c_int
    lib.ref_get_body.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
    return lib


class RefSolver:
    """One reference CollisionSolver3d with persistent trees and point state."""

    def __init__(self, scene, record=True, snap_vel=False):
        self.lib = load()
        s = scene
        self.scene = s
        self._keep = [np.ascontiguousarray(s.tris, dtype=np.int32),
                      np.ascontiguousarray(s.tri_surf, dtype=np.int32),
                      np.ascontiguousarray(s.tri_rest, dtype=np.float64),
                      np.ascontiguousarray(s.bonds, dtype=np.int32),
                      np.ascontiguousarray(s.bond_curve, dtype=np.int32),
                      np.ascontiguousarray(s.bond_rest, dtype=np.float64),
                      np.ascontiguousarray(s.fixed, dtype=np.uint8)]
        t, ts, tr, b, bc, br, fx = self._keep
        self.h = self.lib.ref_create(s.nv, s.nt, _ptr(t, _ip), _ptr(ts, _ip), _ptr(tr, _dp),
                                     s.nb, _ptr(b, _ip), _ptr(bc, _ip), _ptr(br, _dp), _ptr(fx, _up))
        self.lib.ref_set_recording(self.h, int(record), int(snap_vel))
        for sid, b in sorted(scene.bodies.items()):
            com = np.ascontiguousarray(b["com"], dtype=np.float64)
            comv = np.ascontiguousarray(b["comv"], dtype=np.float64)
            if self.lib.ref_set_body(self.h, int(sid), float(b["mass"]), _ptr(com, _dp), _ptr(comv, _dp)):
                raise ValueError(f"no surface {sid}")

    def body(self, surf: int):
        """(centre of mass, centre-of-mass velocity) of a movable body."""
        com, comv = np.zeros(3), np.zeros(3)
        if self.lib.ref_get_body(self.h, int(surf), _ptr(com, _dp), _ptr(comv, _dp)):
            raise ValueError(f"no surface {surf}")
        return com, comv

    def close(self):
        if self.h:
            self.lib.ref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, x_old, x_cand, vel, has_collsn, params=None, domain=None, quiet=True):
        s = self.scene
        x_old = np.ascontiguousarray(x_old, dtype=np.float64)
        x_cand = np.ascontiguousarray(x_cand, dtype=np.float64)
        vel = np.array(vel, dtype=np.float64, copy=True)
        hc = np.array(has_collsn, dtype=np.uint8, copy=True)
        params = s.param_vec() if params is None else np.asarray(params, dtype=np.float64)
        domain = s.domain if domain is None else np.asarray(domain, dtype=np.float64)
        x_out = np.zeros_like(x_old)
        avg = np.zeros_like(x_old)
        hcol = C.c_int(0)
        zr = np.zeros(s.nv, dtype=np.int32)
        rc = self.lib.ref_step(self.h, _ptr(x_old, _dp), _ptr(x_cand, _dp), _ptr(vel, _dp),
                               _ptr(hc, _up), _ptr(params, _dp), _ptr(domain, _dp), int(quiet),
                               _ptr(x_out, _dp), _ptr(avg, _dp), C.byref(hcol), _ptr(zr, _ip))
        return dict(rc=rc, x=x_out, v=vel, has_collsn=hc, avgvel=avg,
                    has_collision=hcol.value, zone_root=zr)

    def passes(self):
        n = self.lib.ref_num_passes(self.h)
        out = np.zeros(n, dtype=np.int32)
        if n:
            self.lib.ref_pass_kinds(self.h, _ptr(out, _ip))
        return out

    def pairs(self):
        n = self.lib.ref_num_pairs(self.h)
        out = np.zeros((n, 11), dtype=np.int32)
        if n:
            self.lib.ref_pairs(self.h, _ptr(out, _ip))
        return out

    def vel_snaps(self):
        n = self.lib.ref_num_vel_snaps(self.h)
        out = np.zeros((n, self.scene.nv, 3), dtype=np.float64)
        if n:
            self.lib.ref_vel_snaps(self.h, _ptr(out, _dp))
        return out
