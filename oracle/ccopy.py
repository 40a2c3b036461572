"""ctypes binding to the C restatement oracle (oracle/cc_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the collision_gb300 package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libcc_oracle.so")
SRC = os.path.join(HERE, "cc_oracle.c")
# Contraction off and round-to-nearest assumed throughout, as for the
# reference build (Makefile:1, 27-28 plus -ffp-contract=off).
CFLAGS = ["-O2", "-std=c99", "-ffp-contract=off", "-frounding-math", "-fPIC", "-shared"]

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_up = C.POINTER(C.c_ubyte)
_lp = C.POINTER(C.c_longlong)


class PairRec(C.Structure):
    _fields_ = [("pass_", C.c_int), ("kind", C.c_int), ("a", C.c_int), ("b", C.c_int),
                ("status", C.c_int), ("dcount", C.c_int * 6)]


class ContactRec(C.Structure):
    _fields_ = [("pass_", C.c_int), ("kind", C.c_int), ("a", C.c_int), ("b", C.c_int),
                ("subtest", C.c_int), ("v", C.c_int * 4)]


CR_SRC = os.path.join(HERE, "cc_oracle_crmath.cpp")
CR_HDR = os.path.join(os.path.dirname(HERE), "collision_gb300", "csrc", "cc_crmath.cuh")
CR_LIB_PATH = os.path.join(BUILD_DIR, "libcc_oracle_cr.so")


def _fresh(lib: str, deps) -> bool:
    return os.path.exists(lib) and os.path.getmtime(lib) >= max(os.path.getmtime(d) for d in deps)


def build(force: bool = False) -> str:
    """Compile the oracle with the host C compiler (seconds), and its
    CCO_CRMATH build, whose acos/cos/sin/pow are correctly rounded."""
    hdr = os.path.join(HERE, "cc_oracle.h")
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or not _fresh(LIB_PATH, [SRC, hdr]):
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", *CFLAGS, "-o", tmp, SRC, "-lm"])
        os.replace(tmp, LIB_PATH)
    if force or not _fresh(CR_LIB_PATH, [SRC, hdr, CR_SRC, CR_HDR]):
        tmp = CR_LIB_PATH + f".tmp{os.getpid()}"
        obj_c, obj_cpp = tmp + ".c.o", tmp + ".cpp.o"
        flags = [f for f in CFLAGS if f != "-shared"]
        subprocess.check_call(["gcc", *flags, "-DCCO_CRMATH", "-c", SRC, "-o", obj_c])
        subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-fPIC", "-c", CR_SRC, "-o", obj_cpp])
        subprocess.check_call(["g++", "-shared", "-Wl,-Bsymbolic", "-o", tmp, obj_c, obj_cpp, "-lm"])
        os.remove(obj_c)
        os.remove(obj_cpp)
        os.replace(tmp, CR_LIB_PATH)
    return LIB_PATH


_LIBS = {}


def load(crmath: bool = False):
    """The oracle library; crmath: its build with correctly rounded
    acos/cos/sin/pow."""
    if crmath in _LIBS:
        return _LIBS[crmath]
    build()
    lib = C.CDLL(CR_LIB_PATH if crmath else LIB_PATH)
    lib.cco_create.restype = C.c_void_p
    lib.cco_create.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, C.c_int, _ip, _dp, _up]
    lib.cco_destroy.argtypes = [C.c_void_p]
    lib.cco_set_recording.argtypes = [C.c_void_p, C.c_int]
    lib.cco_set_zone_cap.argtypes = [C.c_void_p, C.c_int]
    lib.cco_step.restype = C.c_int
    lib.cco_step.argtypes = [C.c_void_p, _dp, _dp, _dp, _up, _dp, _dp, _dp, _dp, _ip, _ip]
    for f in ("cco_num_passes", "cco_num_pairs", "cco_num_contacts", "cco_num_vel_snaps"):
        getattr(lib, f).restype = C.c_int
        getattr(lib, f).argtypes = [C.c_void_p]
    lib.cco_pass_kinds.argtypes = [C.c_void_p, _ip]
    lib.cco_pairs.restype = C.POINTER(PairRec)
    lib.cco_pairs.argtypes = [C.c_void_p]
    lib.cco_contacts.restype = C.POINTER(ContactRec)
    lib.cco_contacts.argtypes = [C.c_void_p]
    lib.cco_vel_snaps.restype = _dp
    lib.cco_vel_snaps.argtypes = [C.c_void_p]
    lib.cco_leaf_rank.restype = C.c_int
    lib.cco_leaf_rank.argtypes = [C.c_void_p, C.c_int, _ip]
    lib.cco_counters.argtypes = [C.c_void_p, _lp]
    lib.cco_check_ccd.restype = C.c_longlong
    lib.cco_check_ccd.argtypes = [C.c_void_p, _dp, _dp, _dp]
    lib.cco_set_body.restype = C.c_int
    lib.cco_set_body.argtypes = [C.c_void_p, C.c_int, C.c_double, _dp, _dp]
    lib.cco_get_body.restype = C.c_int
    lib.cco_get_body.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
    _LIBS[crmath] = lib
    return lib


def _ptr(a, t):
    return a.ctypes.data_as(t) if a is not None else None


REC_PAIRS, REC_CONTACTS, REC_SNAPS = 1, 2, 4


class OracleSolver:
    """One CPU oracle solver: persistent trees and point state, like one
    reference CollisionSolver3d driven by the reference's host loop."""

    def __init__(self, scene, record: int = REC_PAIRS | REC_CONTACTS, crmath: bool = False):
        self.lib = load(crmath)
        s = scene
        self.scene = s
        self._keep = [np.ascontiguousarray(s.tris, dtype=np.int32),
                      np.ascontiguousarray(s.tri_surf, dtype=np.int32),
                      np.ascontiguousarray(s.tri_rest, dtype=np.float64),
                      np.ascontiguousarray(s.bonds, dtype=np.int32),
                      np.ascontiguousarray(s.bond_rest, dtype=np.float64),
                      np.ascontiguousarray(s.fixed, dtype=np.uint8)]
        t, ts, tr, b, br, fx = self._keep
        self.h = self.lib.cco_create(s.nv, s.nt, _ptr(t, _ip), _ptr(ts, _ip), _ptr(tr, _dp),
                                     s.nb, _ptr(b, _ip), _ptr(br, _dp), _ptr(fx, _up))
        if not self.h:
            raise ValueError("oracle rejected the mesh")
        self.lib.cco_set_recording(self.h, int(record))
        for sid, b in sorted(scene.bodies.items()):
            self.set_body(sid, b["mass"], b["com"], b["comv"])

    def set_body(self, surf: int, mass: float, com, comv):
        com = np.ascontiguousarray(com, dtype=np.float64)
        comv = np.ascontiguousarray(comv, dtype=np.float64)
        if self.lib.cco_set_body(self.h, int(surf), float(mass), _ptr(com, _dp), _ptr(comv, _dp)):
            raise ValueError(f"no surface {surf}")

    def body(self, surf: int):
        """(centre of mass, centre-of-mass velocity) of a movable body."""
        com, comv = np.zeros(3), np.zeros(3)
        if self.lib.cco_get_body(self.h, int(surf), _ptr(com, _dp), _ptr(comv, _dp)):
            raise ValueError(f"no surface {surf}")
        return com, comv

    def close(self):
        if getattr(self, "h", None):
            self.lib.cco_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_zone_cap(self, cap: int):
        self.lib.cco_set_zone_cap(self.h, int(cap))

    def step(self, x_old, x_cand, vel, has_collsn, params=None, domain=None):
        s = self.scene
        x_old = np.ascontiguousarray(x_old, dtype=np.float64)
        x_cand = np.ascontiguousarray(x_cand, dtype=np.float64)
        vel = np.array(vel, dtype=np.float64, copy=True)
        hc = np.array(has_collsn, dtype=np.uint8, copy=True)
        params = s.param_vec() if params is None else np.ascontiguousarray(params, dtype=np.float64)
        domain = s.domain if domain is None else np.ascontiguousarray(domain, dtype=np.float64)
        x_out = np.zeros_like(x_old)
        avg = np.zeros_like(x_old)
        hcol = C.c_int(0)
        zr = np.zeros(s.nv, dtype=np.int32)
        rc = self.lib.cco_step(self.h, _ptr(x_old, _dp), _ptr(x_cand, _dp), _ptr(vel, _dp),
                               _ptr(hc, _up), _ptr(params, _dp), _ptr(domain, _dp),
                               _ptr(x_out, _dp), _ptr(avg, _dp), C.byref(hcol), _ptr(zr, _ip))
        return dict(rc=rc, x=x_out, v=vel, has_collsn=hc, avgvel=avg,
                    has_collision=hcol.value, zone_root=zr)

    def check_ccd(self, x_old, x_new, params=None):
        """Element pairs that still collide over [x_old, x_new] by the
        reference's CCD predicate (the exact re-check of a finished step)."""
        x_old = np.ascontiguousarray(x_old, dtype=np.float64)
        x_new = np.ascontiguousarray(x_new, dtype=np.float64)
        params = self.scene.param_vec() if params is None else np.ascontiguousarray(params, dtype=np.float64)
        n = self.lib.cco_check_ccd(self.h, _ptr(x_old, _dp), _ptr(x_new, _dp), _ptr(params, _dp))
        if n < 0:
            raise RuntimeError(f"oracle CCD check failed: {n}")
        return int(n)

    def passes(self):
        n = self.lib.cco_num_passes(self.h)
        out = np.zeros(n, dtype=np.int32)
        if n:
            self.lib.cco_pass_kinds(self.h, _ptr(out, _ip))
        return out

    def pairs(self):
        n = self.lib.cco_num_pairs(self.h)
        if n == 0:
            return np.zeros((0, 11), dtype=np.int32)
        p = self.lib.cco_pairs(self.h)
        arr = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_int)), shape=(n * 11,))
        return arr.reshape(n, 11).copy()

    def contacts(self):
        n = self.lib.cco_num_contacts(self.h)
        if n == 0:
            return np.zeros((0, 9), dtype=np.int32)
        p = self.lib.cco_contacts(self.h)
        arr = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_int)), shape=(n * 9,))
        return arr.reshape(n, 9).copy()

    def vel_snaps(self):
        n = self.lib.cco_num_vel_snaps(self.h)
        if n == 0:
            return np.zeros((0, self.scene.nv, 3))
        p = self.lib.cco_vel_snaps(self.h)
        return np.ctypeslib.as_array(p, shape=(n * self.scene.nv * 3,)).reshape(n, self.scene.nv, 3).copy()

    def leaf_rank(self, which: int):
        out = np.zeros(self.scene.ne, dtype=np.int32)
        ok = self.lib.cco_leaf_rank(self.h, int(which), _ptr(out, _ip))
        return out if ok else None

    def counters(self):
        out = np.zeros(7, dtype=np.int64)
        self.lib.cco_counters(self.h, _ptr(out, _lp))
        return dict(zip(("passes", "prox_pairs", "ccd_pairs", "contacts", "zone_iters",
                         "strain_passes", "rebuilds"), out.tolist()))


def zone_labels(zone_root: np.ndarray) -> np.ndarray:
    """Canonical zone label per point: the smallest point index of its zone."""
    zr = np.asarray(zone_root)
    lab = np.arange(len(zr))
    mins = {}
    for i, r in enumerate(zr):
        mins[r] = min(mins.get(r, i), i)
    for i, r in enumerate(zr):
        lab[i] = mins[r]
    return lab
