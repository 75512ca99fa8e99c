"""ctypes binding of libxdem_gb300.so (the C-ABI of include/xdem_c.h).

The library is the only compute path: if it is missing this module raises,
it never falls back to anything else.
"""
import ctypes as C
import os
import re

from . import types as T

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libxdem_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "xdem_c.h")

_lib = None

vp = C.c_void_p
u32 = C.c_uint
i32 = C.c_int
f64 = C.c_double

_SIGS = {
    "xdem_version": ([], C.c_char_p),
    "xdem_set_stream": ([vp], i32),
    "xdem_last_status": ([], i32),
    "xdem_take_device_status": ([], i32),
    "xdem_set_body_force_buffers": ([vp] * 6, i32),
    "xdem_get_body_force_buffers": ([vp], i32),
    "xdem_last_body_wrench": ([vp], i32),
    "xdem_set_velocity_compat": ([i32], i32),
    "xdem_set_rolling_inertia": ([i32], i32),
    "setDEMSymbolicParameter": ([vp], i32),
    "vv_update_position": ([vp] * 6 + [u32], i32),
    "vv_update_velocity": ([vp] * 9 + [u32], i32),
    "cu_calculateHashAndIndex": ([vp, vp, vp, u32, u32], i32),
    "cu_calculateHashAndIndexForPolygonSphere": ([vp, vp, u32, u32, vp], i32),
    "cu_reorderDataAndFindCellStart": ([vp] * 5 + [u32, u32], i32),
    "cu_reorderDataAndFindCellStart_noalloc": ([vp] * 5 + [u32, u32], i32),
    "cu_calculate_p2p": ([vp] * 16 + [u32], i32),
    "cu_plane_contact_force": ([vp] * 15 + [u32], i32),
    "cu_particle_polygonObject_collision": ([vp] * 19 + [u32, u32], i32),
    "cu_decide_rolling_friction_moment": ([vp] * 6 + [u32], i32),
    "reduction": ([vp, u32], f64),
    "cu_update_meshObjectData": ([vp] * 5 + [u32], i32),
    "cu_clusters_contact": ([vp] * 18 + [u32], i32),
    "cu_cluster_plane_contact": ([vp] * 17 + [u32], i32),
    "cu_cylinder_contact_force": ([vp] * 15 + [u32], i32),
    "cu_cluster_cylinder_contact": ([vp] * 17 + [u32], i32),
    "cu_cluster_meshes_contact": ([vp] * 20 + [u32, u32], i32),
    "cu_decide_cluster_rolling_friction_moment": ([vp] * 7 + [u32], i32),
    "vv_update_cluster_position": ([vp] * 9 + [u32], i32),
    "vv_update_cluster_velocity": ([vp] * 12 + [u32], i32),
    "xdem_sim_create": ([vp, vp], i32),
    "xdem_sim_destroy": ([vp], i32),
    "xdem_sim_set_state": ([vp] * 9, i32),
    "xdem_sim_set_clusters": ([vp, vp, vp, u32, vp, u32], i32),
    "xdem_sim_set_pp_contact": ([vp, vp], i32),
    "xdem_sim_set_scenes": ([vp, u32, vp, vp, vp], i32),
    "xdem_sim_scene_energy": ([vp, vp, vp], i32),
    "xdem_sim_add_plane": ([vp] * 5, i32),
    "xdem_sim_add_cylinder": ([vp] * 5, i32),
    "xdem_sim_add_mesh": ([vp, u32, vp, vp, vp, vp], i32),
    "xdem_sim_get_mesh": ([vp, i32, vp, vp, vp], i32),
    "xdem_sim_set_body": ([vp, i32, vp, vp], i32),
    "xdem_sim_step": ([vp, u32], i32),
    "xdem_sim_body_wrench": ([vp, i32, vp], i32),
    "xdem_sim_set_bodies": ([vp, i32, vp, vp, vp], i32),
    "xdem_sim_body_wrenches": ([vp, i32, vp, vp], i32),
    "xdem_sim_get_state": ([vp] * 8, i32),
    "xdem_sim_get_pairs": ([vp, i32, vp, vp, vp], i32),
    "xdem_sim_set_pairs": ([vp, i32, vp, vp, vp], i32),
    "xdem_sim_energy": ([vp, vp, vp], i32),
    "xdem_sim_status": ([vp], i32),
    "xdem_sim_set_rolling_inertia": ([vp, i32], i32),
    "xdem_sim_set_stream": ([vp, vp], i32),
    "xdem_sim_set_profiling": ([vp, i32], i32),
    "xdem_sim_set_graph": ([vp, i32], i32),
    "xdem_sim_set_persistent": ([vp, i32, C.c_ulonglong], i32),
    "xdem_sim_profile": ([vp, vp, vp, vp], i32),
    "xdem_sim_set_tune": ([vp, vp], i32),
    "xdem_sim_get_tune": ([vp, vp], i32),
    "xdem_sim_autotune": ([vp, u32, vp, vp, vp], i32),
    "xdem_sim_list_rebuilds": ([vp, vp], i32),
    "xdem_sim_save_part": ([vp, C.c_char_p, f64], i32),
    "xdem_sim_load_part": ([vp, C.c_char_p, vp], i32),
    "xdem_adj_create": ([vp, u32, vp], i32),
    "xdem_adj_destroy": ([vp], i32),
    "xdem_adj_forward": ([vp, u32], i32),
    "xdem_adj_backward": ([vp] * 6, i32),
    "xdem_adj_tangent": ([vp, u32, vp, vp, vp], i32),
    "xdem_adj_info": ([vp, vp, vp, vp], i32),
    "xdem_mbd_create": ([f64, f64, vp, vp], i32),
    "xdem_mbd_destroy": ([vp], i32),
    "xdem_mbd_set_tolerance": ([vp, f64], i32),
    "xdem_mbd_add_body": ([vp, f64, vp, vp, vp, vp, vp, vp], i32),
    "xdem_mbd_add_revolute": ([vp, i32, i32, vp, vp, vp], i32),
    "xdem_mbd_add_translational": ([vp, i32, i32, vp, vp, vp], i32),
    "xdem_mbd_add_rotation_driver": ([vp, i32, f64], i32),
    "xdem_mbd_initialize": ([vp], i32),
    "xdem_mbd_set_contact_wrench": ([vp, i32, vp], i32),
    "xdem_mbd_step": ([vp, vp], i32),
    "xdem_mbd_get_body": ([vp, i32, vp, vp, vp], i32),
    "xdem_mbd_body_record": ([vp, i32, vp], i32),
    "xdem_mbd_info": ([vp, vp, vp, vp], i32),
    "xdem_mbd_multipliers": ([vp, vp, i32], i32),
}


def header_symbols(path=HEADER):
    """Every function the public header declares with XDEM_API."""
    src = open(path).read()
    return re.findall(r"XDEM_API\s+[\w\s\*]+?\b(\w+)\s*\(", src)


def lib():
    """Loads the library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with xdynamics_dll_gb300.build.build() "
                           "(or __graft_entry__.build()); there is no fallback path")
    L = C.CDLL(LIB_PATH)
    for name, (args, res) in _SIGS.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


class XdemError(RuntimeError):
    pass


def check(status, what=""):
    if status != 0:
        names = [n for n in dir(T) if n.startswith("XDEM_ERR_") and status & getattr(T, n)]
        raise XdemError(f"{what}: status {status:#x} {names}")
    return status
