"""ctypes mirrors of the structs in include/xdem_c.h.

Each struct is byte-compatible with its reference counterpart in
include/xdynamics_parallel/xParallelDEM_decl.cuh (decl:128-243) and
include/xTypes.h:263, so an array of them can be filled on the host and
copied to the device as the reference's contact objects do.
"""
import ctypes as C

import numpy as np

MAX_P2P_COUNT = 12
MAX_P2PL_COUNT = 3
MAX_P2CY_COUNT = 3
MAX_P2MS_COUNT = 5
DEVICE_BODY_MEM_SIZE = 120

# body record layout (decl:20)
MM, PX, PY, PZ, VX, VY, VZ, E0, E1, E2, E3, ED0, ED1, ED2, ED3 = range(15)

XDEM_OK = 0
XDEM_ERR_P2P_OVERFLOW = 1 << 0
XDEM_ERR_P2PL_OVERFLOW = 1 << 1
XDEM_ERR_P2MS_OVERFLOW = 1 << 2
XDEM_ERR_TRI_CANDIDATES = 1 << 3
XDEM_ERR_NONFINITE = 1 << 4
XDEM_ERR_P2CY_OVERFLOW = 1 << 5
XDEM_ERR_BARRIER = 1 << 6
XDEM_ERR_CUDA = 1 << 8
XDEM_ERR_ARG = 1 << 9
XDEM_ERR_NOT_SET = 1 << 10
XDEM_ERR_ALLOC = 1 << 11

XDEM_FP64 = 0
XDEM_MIXED = 1


class Double3(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]


class UInt3(C.Structure):
    _fields_ = [("x", C.c_uint), ("y", C.c_uint), ("z", C.c_uint)]


class DemParameters(C.Structure):
    """device_dem_parameters (decl:128-150)."""
    _fields_ = [
        ("rollingCondition", C.c_bool),
        ("contact_model", C.c_int),
        ("np", C.c_uint),
        ("nmp", C.c_uint),
        ("nCluster", C.c_uint),
        ("nClusterObject", C.c_uint),
        ("nTsdaConnection", C.c_uint),
        ("nTsdaConnectionList", C.c_uint),
        ("nTsdaConnectionBodyData", C.c_uint),
        ("nsphere", C.c_uint),
        ("nplane", C.c_uint),
        ("ncylinder", C.c_uint),
        ("ncell", C.c_uint),
        ("grid_size", UInt3),
        ("dt", C.c_double),
        ("half2dt", C.c_double),
        ("cell_size", C.c_double),
        ("cohesion", C.c_double),
        ("gravity", Double3),
        ("world_origin", Double3),
    ]


class TriangleInfo(C.Structure):
    """device_triangle_info (decl:152-159)."""
    _fields_ = [("id", C.c_int), ("tid", C.c_uint), ("P", Double3), ("Q", Double3), ("R", Double3)]


class PlaneInfo(C.Structure):
    """device_plane_info (decl:161-174)."""
    _fields_ = [("id", C.c_uint), ("l1", C.c_double), ("l2", C.c_double)] + [
        (n, Double3) for n in ("u1", "u2", "uw", "xw", "pa", "pb", "w2", "w3", "w4")
    ]


class ContactProperty(C.Structure):
    """device_contact_property (decl:230-243), xContact.cpp:308-312 order."""
    _fields_ = [(n, C.c_double) for n in
                ("Ei", "Ej", "pri", "prj", "Gi", "Gj", "rest", "fric", "s_fric",
                 "rfric", "coh", "sratio", "amp")]


class CylinderInfo(C.Structure):
    """device_cylinder_info (decl:220-228)."""
    _fields_ = [("id", C.c_uint), ("empty_part", C.c_uint), ("thickness", C.c_double), ("len_rr", Double3),
                ("pbase", Double3), ("ptop", Double3)]


class ClusterInformation(C.Structure):
    """xClusterInformation (include/xTypes.h:263)."""
    _fields_ = [("sid", C.c_uint), ("scid", C.c_uint), ("count", C.c_uint), ("neach", C.c_uint)]


class Tune(C.Structure):
    """xdem_tune (include/xdem_c.h): block shapes of the mixed contact stage."""
    _fields_ = [("nt_pairs", C.c_uint), ("stage", C.c_uint), ("nt_bodies", C.c_uint), ("occ_pairs", C.c_uint),
                ("occ_bodies", C.c_uint), ("skin_div", C.c_uint), ("contact_ms", C.c_double)]
    SHAPE = ("nt_pairs", "stage", "nt_bodies", "occ_pairs", "occ_bodies", "skin_div")

    def as_dict(self):
        d = {k: getattr(self, k) for k in self.SHAPE}
        d["contact_ms"] = self.contact_ms
        return d


class SimConfig(C.Structure):
    """xdem_sim_config (include/xdem_c.h)."""
    _fields_ = [
        ("np", C.c_uint),
        ("ns", C.c_uint),
        ("precision", C.c_int),
        ("contact_model", C.c_int),
        ("velocity_compat", C.c_int),
        ("dt", C.c_double),
        ("gravity", C.c_double * 3),
        ("world_origin", C.c_double * 3),
        ("cell_size", C.c_double),
        ("grid_size", C.c_uint * 3),
        ("launcher_path", C.c_int),
    ]


assert C.sizeof(DemParameters) == 144
assert C.sizeof(PlaneInfo) == 240
assert C.sizeof(TriangleInfo) == 80
assert C.sizeof(ContactProperty) == 104
assert C.sizeof(ClusterInformation) == 16


def d3(v):
    return Double3(float(v[0]), float(v[1]), float(v[2]))


def make_params(*, np_, dt, gravity=(0.0, -9.80665, 0.0), cell_size, grid=(128, 128, 128),
                origin=(-1.0, -1.0, -1.0), contact_model=1, ncluster=0, nco=0, nplane=0, ncylinder=0):
    p = DemParameters()
    p.rollingCondition = False
    p.contact_model = contact_model
    p.np = np_
    p.nCluster = ncluster
    p.nClusterObject = nco
    p.nplane = nplane
    p.ncylinder = ncylinder
    p.ncell = grid[0] * grid[1] * grid[2]
    p.grid_size = UInt3(*grid)
    p.dt = dt
    p.half2dt = 0.5 * dt * dt
    p.cell_size = cell_size
    p.cohesion = 0.0
    p.gravity = d3(gravity)
    p.world_origin = d3(origin)
    return p


def make_contact_property(*, E_i, E_j, nu_i, nu_j, rest, fric, s_fric=None, rfric=0.0,
                          coh=0.0, sratio=0.0, amp=1.0):
    G_i = E_i / (2.0 * (1.0 + nu_i))
    G_j = E_j / (2.0 * (1.0 + nu_j))
    return ContactProperty(E_i, E_j, nu_i, nu_j, G_i, G_j, rest, fric,
                           fric if s_fric is None else s_fric, rfric, coh, sratio, amp)


def plane_from_points(pid, xw, w2, w4):
    """Finite rectangle with corner xw and edges xw->w2, xw->w4, the frame of
    xParticlePlaneContact::update (xParticlePlaneContact.cpp:96-111):
    u1, u2 along the edges, uw = u1 x u2 (the side particles touch)."""
    xw = np.asarray(xw, float)
    w2 = np.asarray(w2, float)
    w4 = np.asarray(w4, float)
    pa = w2 - xw
    pb = w4 - xw
    l1 = float(np.sqrt(pa @ pa))
    l2 = float(np.sqrt(pb @ pb))
    u1 = pa / l1
    u2 = pb / l2
    uw = np.cross(u1, u2)
    w3 = xw + pa + pb
    p = PlaneInfo()
    p.id = pid
    p.l1, p.l2 = l1, l2
    p.u1, p.u2, p.uw = d3(u1), d3(u2), d3(uw)
    p.xw, p.pa, p.pb = d3(xw), d3(pa), d3(pb)
    p.w2, p.w3, p.w4 = d3(w2), d3(w3), d3(w4)
    return p


def cube_planes(pmin, pmax, first_id=0):
    """Six planes of an axis-aligned box, in the order and orientation of
    xCubeObject::define (xCubeObject.cpp:45-65): each uses the
    define(xw, pa, pb) form, so w2 = pa, w4 = pb."""
    mn = np.asarray(pmin, float)
    mx = np.asarray(pmax, float)
    sx = float(np.linalg.norm(mx - np.array([mn[0], mx[1], mx[2]])))
    sy = float(np.linalg.norm(mx - np.array([mx[0], mn[1], mx[2]])))
    sz = float(np.linalg.norm(mx - np.array([mx[0], mx[1], mn[2]])))
    X, Y, Z = np.array([sx, 0, 0]), np.array([0, sy, 0]), np.array([0, 0, sz])
    defs = [
        (mn, mn + Z, mn + X),
        (mn, mn + Y, mn + Z),
        (mn + X, mn + X + Z, mn + X + Y),
        (mn, mn + X, mn + Y),
        (mn + Z, mn + Y + Z, mn + X + Z),
        (mn + Y, mn + X + Y, mn + Y + Z),
    ]
    return [plane_from_points(first_id + i, *d) for i, d in enumerate(defs)]


def body_record(mass=0.0, pos=(0.0, 0.0, 0.0), vel=(0.0, 0.0, 0.0),
                ep=(1.0, 0.0, 0.0, 0.0), ed=(0.0, 0.0, 0.0, 0.0)):
    """The 15-double record of xParticlePlaneContact.cpp:117-125."""
    return np.array([mass, *pos, *vel, *ep, *ed], dtype=np.float64)
