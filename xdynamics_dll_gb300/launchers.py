"""Launcher surface from Python: every reference-named launcher of
include/xdem_c.h called through ctypes on device mirrors of host arrays.

`Launchers` keeps one device copy per host numpy array (or ctypes struct /
array) it is given, uploads on first use and copies everything back with
download().  Device memory comes from torch; all compute is the library's.
"""
import ctypes as C

import numpy as np

from . import _lib
from . import types as T


class Launchers:
    def __init__(self, device="cuda"):
        import torch
        self.torch = torch
        self.device = device
        self.L = _lib.lib()
        self.mirrors = {}   # id(host) -> (host, tensor)
        self.prm = None

    # ------------------------------------------------------------ memory
    def d(self, a):
        """Device pointer of the mirror of host object `a` (uploads on first use)."""
        if a is None:
            return None
        key = id(a)
        m = self.mirrors.get(key)
        if m is None:
            torch = self.torch
            if isinstance(a, np.ndarray):
                t = torch.from_numpy(np.ascontiguousarray(a)).to(self.device)
            else:  # ctypes struct or array
                raw = np.frombuffer(C.string_at(C.addressof(a), C.sizeof(a)), dtype=np.uint8).copy()
                t = torch.from_numpy(raw).to(self.device)
            m = (a, t)
            self.mirrors[key] = m
        return C.c_void_p(m[1].data_ptr())

    def download(self):
        self.torch.cuda.synchronize()
        for a, t in self.mirrors.values():
            if isinstance(a, np.ndarray):
                a[...] = t.cpu().numpy().reshape(a.shape)
            else:
                raw = t.cpu().numpy().tobytes()
                C.memmove(C.addressof(a), raw, len(raw))

    def forget(self):
        self.mirrors.clear()

    def _ck(self, r, what):
        return _lib.check(r, what)

    # ------------------------------------------------------------ launchers
    def set_params(self, prm):
        self.prm = prm
        self._ck(self.L.setDEMSymbolicParameter(C.byref(prm)), "setDEMSymbolicParameter")

    def set_velocity_compat(self, on):
        self.L.xdem_set_velocity_compat(int(on))

    def vv_pos(self, s):
        self._ck(self.L.vv_update_position(self.d(s["pos"]), self.d(s["ep"]), self.d(s["vel"]), self.d(s["ev"]),
                                           self.d(s["acc"]), self.d(s["ea"]), s["np"]), "vv_update_position")

    def vv_vel(self, s, compat):
        self.set_velocity_compat(compat)
        self._ck(self.L.vv_update_velocity(self.d(s["vel"]), self.d(s["acc"]), self.d(s["ep"]), self.d(s["ev"]),
                                           self.d(s["ea"]), self.d(s["force"]), self.d(s["moment"]),
                                           self.d(s["mass"]), self.d(s["inertia"]), s["np"]),
                 "vv_update_velocity")

    def hash(self, g, pos, sid, n):
        self._ck(self.L.cu_calculateHashAndIndex(self.d(g["hash"]), self.d(g["index"]), self.d(pos), sid, n),
                 "cu_calculateHashAndIndex")
        return 0

    def reorder(self, g, n):
        self._ck(self.L.cu_reorderDataAndFindCellStart(self.d(g["hash"]), self.d(g["index"]), self.d(g["cstart"]),
                                                       self.d(g["cend"]), self.d(g["sorted_index"]), n,
                                                       g["cstart"].size), "cu_reorderDataAndFindCellStart")

    def _status(self):
        return self.L.xdem_take_device_status()

    def p2p(self, s, g, cp):
        self._ck(self.L.cu_calculate_p2p(self.d(s["pos"]), self.d(s["ep"]), self.d(s["vel"]), self.d(s["ev"]),
                                         self.d(s["force"]), self.d(s["moment"]), self.d(s["mass"]),
                                         self.d(s["tmax"]), self.d(s["rres"]), self.d(s["pp_count"]),
                                         self.d(s["pp_id"]), self.d(s["pp_tsd"]), self.d(g["sorted_index"]),
                                         self.d(g["cstart"]), self.d(g["cend"]), self.d(cp), s["np"]),
                 "cu_calculate_p2p")
        return self._status()

    def _bf(self, s):
        self.L.xdem_set_body_force_buffers(*[self.d(b) for b in s["bf"]])

    def plane(self, s, plane, dbi, cp):
        self._bf(s)
        self._ck(self.L.cu_plane_contact_force(self.d(plane), self.d(dbi), self.d(cp), self.d(s["pos"]),
                                               self.d(s["ep"]), self.d(s["vel"]), self.d(s["ev"]),
                                               self.d(s["force"]), self.d(s["moment"]), self.d(s["mass"]),
                                               self.d(s["tmax"]), self.d(s["rres"]), self.d(s["pl_count"]),
                                               self.d(s["pl_id"]), self.d(s["pl_tsd"]), s["np"]),
                 "cu_plane_contact_force")
        return self._status()

    def last_wrench(self):
        out = np.zeros(6)
        self._ck(self.L.xdem_last_body_wrench(out.ctypes.data_as(C.c_void_p)), "xdem_last_body_wrench")
        return out

    def mesh(self, s, g, dti, dbi, cp, ntri):
        self._bf(s)
        self._ck(self.L.cu_particle_polygonObject_collision(
            self.d(dti), self.d(dbi), self.d(s["pos"]), self.d(s["ep"]), self.d(s["vel"]), self.d(s["ev"]),
            self.d(s["force"]), self.d(s["moment"]), self.d(s["mass"]), self.d(s["tmax"]), self.d(s["rres"]),
            self.d(s["ms_count"]), self.d(s["ms_id"]), self.d(s["ms_tsd"]), self.d(s.get("dsph")),
            self.d(g["sorted_index"]), self.d(g["cstart"]), self.d(g["cend"]), self.d(cp), s["np"], ntri),
            "cu_particle_polygonObject_collision")
        return self._status()

    def rolling(self, s):
        self._ck(self.L.cu_decide_rolling_friction_moment(self.d(s["tmax"]), self.d(s["rres"]),
                                                          self.d(s["inertia"]), self.d(s["ep"]), self.d(s["ev"]),
                                                          self.d(s["moment"]), s["np"]),
                 "cu_decide_rolling_friction_moment")

    def update_mesh(self, dbi, vlist, sphere, dlocal, dti, ntri):
        self._ck(self.L.cu_update_meshObjectData(self.d(vlist), self.d(sphere), self.d(dlocal), self.d(dti),
                                                 self.d(dbi), ntri), "cu_update_meshObjectData")

    def clusters_p2p(self, s, g, cp):
        self._ck(self.L.cu_clusters_contact(self.d(s["pos"]), self.d(s["cpos"]), self.d(s["ep"]), self.d(s["vel"]),
                                            self.d(s["ev"]), self.d(s["force"]), self.d(s["moment"]),
                                            self.d(s["mass"]), self.d(s["tmax"]), self.d(s["rres"]),
                                            self.d(s["pp_count"]), self.d(s["pp_id"]), self.d(s["pp_tsd"]),
                                            self.d(g["sorted_index"]), self.d(g["cstart"]), self.d(g["cend"]),
                                            self.d(cp), self.d(s["xci"]), s["np"]), "cu_clusters_contact")
        return self._status()

    def cluster_plane(self, s, plane, dbi, cp):
        self._bf(s)
        self._ck(self.L.cu_cluster_plane_contact(self.d(plane), self.d(dbi), self.d(cp), self.d(s["pos"]),
                                                 self.d(s["cpos"]), self.d(s["ep"]), self.d(s["vel"]),
                                                 self.d(s["ev"]), self.d(s["force"]), self.d(s["moment"]),
                                                 self.d(s["mass"]), self.d(s["tmax"]), self.d(s["rres"]),
                                                 self.d(s["pl_count"]), self.d(s["pl_id"]), self.d(s["pl_tsd"]),
                                                 self.d(s["xci"]), s["np"]), "cu_cluster_plane_contact")
        return self._status()

    def cylinder(self, s, cyl, bi, cp):
        """cu_cylinder_contact_force, or cu_cluster_cylinder_contact when the
        state has cluster centres (s["cpos"]); pairs in s["cy_count"],
        s["cy_id"], s["cy_tsd"] (MAX_P2CY_COUNT slots a particle)."""
        self._bf(s)
        if s.get("cpos") is None:
            r = self.L.cu_cylinder_contact_force(
                self.d(cyl), self.d(bi), self.d(cp), self.d(s["pos"]), self.d(s["ep"]), self.d(s["vel"]),
                self.d(s["ev"]), self.d(s["force"]), self.d(s["moment"]), self.d(s["mass"]), self.d(s["tmax"]),
                self.d(s["rres"]), self.d(s["cy_count"]), self.d(s["cy_id"]), self.d(s["cy_tsd"]), s["np"])
        else:
            r = self.L.cu_cluster_cylinder_contact(
                self.d(cyl), self.d(bi), self.d(s["xci"]), self.d(cp), self.d(s["pos"]), self.d(s["cpos"]),
                self.d(s["ep"]), self.d(s["vel"]), self.d(s["ev"]), self.d(s["force"]), self.d(s["moment"]),
                self.d(s["mass"]), self.d(s["tmax"]), self.d(s["rres"]), self.d(s["cy_count"]), self.d(s["cy_id"]),
                self.d(s["cy_tsd"]), s["np"])
        self._ck(r, "cu_cylinder_contact_force")
        return self._status()

    def cluster_mesh(self, s, g, dti, dbi, cp, ntri):
        self._bf(s)
        self._ck(self.L.cu_cluster_meshes_contact(
            self.d(dti), self.d(dbi), self.d(s["pos"]), self.d(s["cpos"]), self.d(s["ep"]), self.d(s["vel"]),
            self.d(s["ev"]), self.d(s["force"]), self.d(s["moment"]), self.d(cp), self.d(s["mass"]),
            self.d(s["tmax"]), self.d(s["rres"]), self.d(s["ms_count"]), self.d(s["ms_id"]), self.d(s["ms_tsd"]),
            self.d(g["sorted_index"]), self.d(g["cstart"]), self.d(g["cend"]), self.d(s["xci"]), s["np"], ntri),
            "cu_cluster_meshes_contact")
        return self._status()

    def cluster_rolling(self, s):
        self._ck(self.L.cu_decide_cluster_rolling_friction_moment(
            self.d(s["tmax"]), self.d(s["rres"]), self.d(s["inertia"]), self.d(s["ep"]), self.d(s["ev"]),
            self.d(s["moment"]), self.d(s["xci"]), s["np"]), "cu_decide_cluster_rolling_friction_moment")

    def vv_cluster_pos(self, s):
        self._ck(self.L.vv_update_cluster_position(self.d(s["pos"]), self.d(s["cpos"]), self.d(s["ep"]),
                                                   self.d(s["rloc"]), self.d(s["vel"]), self.d(s["acc"]),
                                                   self.d(s["ev"]), self.d(s["ea"]), self.d(s["xci"]), s["ns"]),
                 "vv_update_cluster_position")

    def vv_cluster_vel(self, s):
        self._ck(self.L.vv_update_cluster_velocity(self.d(s["cpos"]), self.d(s["ep"]), self.d(s["vel"]),
                                                   self.d(s["acc"]), self.d(s["ev"]), self.d(s["ea"]),
                                                   self.d(s["force"]), self.d(s["moment"]), self.d(s["rloc"]),
                                                   self.d(s["mass"]), self.d(s["inertia"]), self.d(s["xci"]),
                                                   s["ns"]), "vv_update_cluster_velocity")

    def reduction(self, a):
        r = self.L.reduction(self.d(a), a.size)
        _lib.check(self.L.xdem_last_status(), "reduction")
        return r
