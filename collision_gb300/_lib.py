"""ctypes binding of the C ABI in include/collision_gb300.h.

Loads the in-tree library collision_gb300/_build/libcollision_gb300.so and
raises if it is missing: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "_build", "libcollision_gb300.so")
HEADER = os.path.join(ROOT, "include", "collision_gb300.h")

STATUS = {0: "CC_OK", 1: "CC_BAD_INPUT", 2: "CC_PAIR_OVERFLOW", 3: "CC_STACK_OVERFLOW", 4: "CC_ITER_CAP",
          5: "CC_NAN_DETECTED", 6: "CC_CUDA_ERROR", 7: "CC_CONTACT_OVERFLOW", 8: "CC_NO_MEMORY"}


class CCError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class cc_params(C.Structure):
    _fields_ = [("dt", C.c_double), ("thickness", C.c_double), ("eps", C.c_double), ("k", C.c_double),
                ("m", C.c_double), ("lam", C.c_double), ("cr", C.c_double)]


class cc_mesh(C.Structure):
    _fields_ = [("n_points", C.c_int32), ("n_tris", C.c_int32), ("tris", C.c_void_p),
                ("tri_surface", C.c_void_p), ("tri_rest_len", C.c_void_p), ("n_bonds", C.c_int32),
                ("bonds", C.c_void_p), ("bond_rest_len", C.c_void_p), ("fixed", C.c_void_p)]


def declared_symbols() -> list[str]:
    """Every function the public header declares."""
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(cc_[a-z_]+)\s*\(", txt)))


_LIB = None


def load(path: str = LIB_PATH):
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise RuntimeError(f"collision_gb300 CUDA library not built ({path}); run "
                           "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(path)
    vp, ip, dp, up, lp = C.c_void_p, C.POINTER(C.c_int), C.c_void_p, C.c_void_p, C.POINTER(C.c_longlong)
    lib.cc_create.restype = C.c_int
    lib.cc_create.argtypes = [C.c_int, C.POINTER(C.c_void_p)]
    lib.cc_destroy.restype = None
    lib.cc_destroy.argtypes = [vp]
    lib.cc_assemble.restype = C.c_int
    lib.cc_assemble.argtypes = [vp, C.POINTER(cc_mesh)]
    lib.cc_set_params.restype = C.c_int
    lib.cc_set_params.argtypes = [vp, C.POINTER(cc_params)]
    lib.cc_set_domain_boundary.restype = C.c_int
    lib.cc_set_domain_boundary.argtypes = [vp, dp, dp]
    lib.cc_assemble_batch.restype = C.c_int
    lib.cc_assemble_batch.argtypes = [vp, C.POINTER(cc_mesh), C.c_int]
    lib.cc_num_scenes.restype = C.c_int
    lib.cc_num_scenes.argtypes = [vp]
    lib.cc_get_scene_offsets.restype = C.c_int
    lib.cc_get_scene_offsets.argtypes = [vp, ip, ip]
    lib.cc_set_scene_params.restype = C.c_int
    lib.cc_set_scene_params.argtypes = [vp, C.c_int, C.POINTER(cc_params)]
    lib.cc_set_scene_domain_boundary.restype = C.c_int
    lib.cc_set_scene_domain_boundary.argtypes = [vp, C.c_int, dp, dp]
    lib.cc_check_ccd.restype = C.c_int
    lib.cc_check_ccd.argtypes = [vp, dp, dp, lp, ip]
    lib.cc_autotune.restype = C.c_int
    lib.cc_autotune.argtypes = [vp, C.POINTER(C.c_double)]
    lib.cc_set_tuning.restype = C.c_int
    lib.cc_set_tuning.argtypes = [vp, C.c_int, C.c_int]
    lib.cc_get_tuning.restype = C.c_int
    lib.cc_get_tuning.argtypes = [vp, C.c_int]
    lib.cc_set_vtk_dump.restype = C.c_int
    lib.cc_set_vtk_dump.argtypes = [vp, C.c_char_p]
    lib.cc_set_zone_cap.restype = C.c_int
    lib.cc_set_zone_cap.argtypes = [vp, C.c_int]
    lib.cc_set_body.restype = C.c_int
    lib.cc_set_body.argtypes = [vp, C.c_int, C.c_int, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.cc_get_body.restype = C.c_int
    lib.cc_get_body.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.cc_get_scene_status.restype = C.c_int
    lib.cc_get_scene_status.argtypes = [vp, ip]
    lib.cc_set_scene_enabled.restype = C.c_int
    lib.cc_set_scene_enabled.argtypes = [vp, C.c_int, C.c_int]
    lib.cc_set_host_threads.restype = C.c_int
    lib.cc_set_host_threads.argtypes = [vp, C.c_int]
    lib.cc_get_scene_pass_kinds.restype = C.c_int
    lib.cc_get_scene_pass_kinds.argtypes = [vp, C.c_int, ip, C.c_int]
    for f in ("cc_resolve", "cc_resolve_device", "cc_resolve_batch", "cc_resolve_batch_device"):
        getattr(lib, f).restype = C.c_int
        getattr(lib, f).argtypes = [vp, dp, dp, dp, up, dp, ip]
    lib.cc_get_counters.restype = C.c_int
    lib.cc_get_counters.argtypes = [vp, lp, C.c_int]
    lib.cc_set_recording.restype = C.c_int
    lib.cc_set_recording.argtypes = [vp, C.c_int]
    lib.cc_get_visits.restype = C.c_int
    lib.cc_get_visits.argtypes = [vp, ip, C.c_int]
    lib.cc_get_pass_kinds.restype = C.c_int
    lib.cc_get_pass_kinds.argtypes = [vp, ip, C.c_int]
    lib.cc_get_zone_roots.restype = C.c_int
    lib.cc_get_zone_roots.argtypes = [vp, ip]
    lib.cc_get_leaf_ranks.restype = C.c_int
    lib.cc_get_leaf_ranks.argtypes = [vp, C.c_int, ip]
    lib.cc_get_tree_volume.restype = C.c_int
    lib.cc_get_tree_volume.argtypes = [vp, C.c_int, C.POINTER(C.c_double)]
    lib.cc_debug_candidate_pairs.restype = C.c_int
    lib.cc_debug_candidate_pairs.argtypes = [vp, C.c_int, C.c_int, ip, C.c_int]
    lib.cc_set_stream.restype = C.c_int
    lib.cc_set_stream.argtypes = [vp, vp]
    lib.cc_set_strain_window.restype = C.c_int
    lib.cc_set_strain_window.argtypes = [vp, C.c_int]
    lib.cc_set_mode.restype = C.c_int
    lib.cc_set_mode.argtypes = [vp, C.c_int]
    lib.cc_set_profiling.restype = C.c_int
    lib.cc_set_profiling.argtypes = [vp, C.c_int]
    lib.cc_get_profile.restype = C.c_int
    lib.cc_get_profile.argtypes = [vp, C.POINTER(C.c_double), lp, C.c_int]
    lib.cc_profile_stage_name.restype = C.c_char_p
    lib.cc_profile_stage_name.argtypes = [C.c_int]
    lib.cc_selftest_math.restype = C.c_int
    lib.cc_selftest_math.argtypes = [C.c_int, C.c_int, dp, dp, dp, C.c_int]
    lib.cc_candidate_pairs_static.restype = C.c_int
    lib.cc_candidate_pairs_static.argtypes = [C.c_int, dp, C.c_int, vp, C.c_int, ip, vp]
    lib.cc_static_last_error.restype = C.c_int
    lib.cc_static_last_error.argtypes = [C.c_char_p, C.c_int]
    lib.cc_last_error.restype = C.c_int
    lib.cc_last_error.argtypes = [vp, C.c_char_p, C.c_int]
    _LIB = lib
    return lib
