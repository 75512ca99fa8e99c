"""Scene handle from Python: xdem_sim_* of include/xdem_c.h.

`Sim(scene)` creates the handle, uploads the scene (state, contact
properties, planes, meshes, clusters) and exposes step / state / pairs /
wrench / energy.  Host arrays use the reference layout.
"""
import ctypes as C

import numpy as np

from . import _lib
from . import types as T


def _p(a):
    return None if a is None else C.c_void_p(np.ascontiguousarray(a).ctypes.data)


class Sim:
    def __init__(self, scene, precision=T.XDEM_FP64, velocity_compat=0, launcher_path=0):
        self.L = _lib.lib()
        self.scene = scene
        cfg = T.SimConfig()
        cfg.np = scene.np_
        cfg.ns = 0 if scene.ns == scene.np_ else scene.ns
        cfg.precision = precision
        cfg.contact_model = scene.contact_model
        cfg.velocity_compat = velocity_compat
        cfg.dt = scene.dt
        for i in range(3):
            cfg.gravity[i] = scene.gravity[i]
            cfg.world_origin[i] = scene.origin[i]
            cfg.grid_size[i] = scene.grid[i]
        cfg.cell_size = scene.cell_size
        cfg.launcher_path = launcher_path
        self.cfg = cfg
        h = C.c_void_p()
        _lib.check(self.L.xdem_sim_create(C.byref(cfg), C.byref(h)), "xdem_sim_create")
        self.h = h
        self._keep = []
        self.set_state(scene.pos, scene.vel, scene.acc, scene.ep, scene.ev, scene.ea, scene.mass, scene.inertia)
        if scene.cpos is not None:
            xci = np.ascontiguousarray(scene.xci, dtype=np.uint32)
            rloc = np.ascontiguousarray(scene.rloc, dtype=np.float64)
            _lib.check(self.L.xdem_sim_set_clusters(h, _p(scene.cpos), _p(xci), xci.size // 4, _p(rloc),
                                                    rloc.size // 3), "xdem_sim_set_clusters")
        if scene.pp_cp is not None:
            _lib.check(self.L.xdem_sim_set_pp_contact(h, C.byref(scene.pp_cp)), "xdem_sim_set_pp_contact")
        self.bodies = []
        for k, pl in enumerate(scene.planes):
            b = C.c_int()
            rec = np.ascontiguousarray(scene.plane_body[k], dtype=np.float64)
            _lib.check(self.L.xdem_sim_add_plane(h, C.byref(pl), _p(rec), C.byref(scene.plane_cp[k]), C.byref(b)),
                       "xdem_sim_add_plane")
            self.bodies.append(b.value)
        for cy in getattr(scene, "cylinders", []):
            b = C.c_int()
            rec = np.ascontiguousarray(cy["body"], dtype=np.float64)
            _lib.check(self.L.xdem_sim_add_cylinder(h, C.byref(cy["cyl"]), _p(rec), C.byref(cy["cp"]), C.byref(b)),
                       "xdem_sim_add_cylinder")
            self.bodies.append(b.value)
        for m in scene.meshes:
            b = C.c_int()
            vl = np.ascontiguousarray(m["vlist_local"], dtype=np.float64).reshape(-1)
            rec = np.ascontiguousarray(m["body"], dtype=np.float64)
            _lib.check(self.L.xdem_sim_add_mesh(h, vl.size // 9, _p(vl), _p(rec), C.byref(m["cp"]), C.byref(b)),
                       "xdem_sim_add_mesh")
            self.bodies.append(b.value)

    def close(self):
        if self.h:
            self.L.xdem_sim_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ state
    def set_state(self, pos, vel, acc, ep, ev, ea, mass, inertia):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) if a is not None else None
                for a in (pos, vel, acc, ep, ev, ea, mass, inertia)]
        _lib.check(self.L.xdem_sim_set_state(self.h, *[_p(a) for a in arrs]), "xdem_sim_set_state")

    def step(self, n=1):
        _lib.check(self.L.xdem_sim_step(self.h, int(n)), "xdem_sim_step")

    def state(self):
        sc = self.scene
        out = dict(pos=np.zeros(sc.np_ * 4), vel=np.zeros(sc.ns * 3), acc=np.zeros(sc.ns * 3),
                   ep=np.zeros(sc.ns * 4), ev=np.zeros(sc.ns * 4), ea=np.zeros(sc.ns * 4))
        cpos = np.zeros(sc.ns * 4) if sc.cpos is not None else None
        _lib.check(self.L.xdem_sim_get_state(self.h, _p(out["pos"]), _p(out["vel"]), _p(out["acc"]), _p(out["ep"]),
                                             _p(out["ev"]), _p(out["ea"]), _p(cpos)), "xdem_sim_get_state")
        if cpos is not None:
            out["cpos"] = cpos
        return out

    def pairs(self, kind):
        """kind 0 particle pairs, 1 planes, 2 triangles, 3 cylinders."""
        cap = [T.MAX_P2P_COUNT, T.MAX_P2PL_COUNT, T.MAX_P2MS_COUNT, T.MAX_P2CY_COUNT][kind]
        n = self.scene.np_
        cnt = np.zeros(n, np.uint32)
        ids = np.zeros(n * cap, np.uint32)
        tsd = np.zeros(n * cap * 2)
        _lib.check(self.L.xdem_sim_get_pairs(self.h, kind, _p(cnt), _p(ids), _p(tsd)), "xdem_sim_get_pairs")
        return cnt, ids, tsd

    def set_pairs(self, kind, cnt, ids, tsd):
        _lib.check(self.L.xdem_sim_set_pairs(self.h, kind, _p(np.ascontiguousarray(cnt, np.uint32)),
                                             _p(np.ascontiguousarray(ids, np.uint32)),
                                             _p(np.ascontiguousarray(tsd, np.float64))), "xdem_sim_set_pairs")

    def mesh(self, body):
        n = C.c_uint()
        _lib.check(self.L.xdem_sim_get_mesh(self.h, body, None, None, C.byref(n)), "xdem_sim_get_mesh")
        tri = (T.TriangleInfo * n.value)()
        sph = np.zeros(n.value * 4)
        _lib.check(self.L.xdem_sim_get_mesh(self.h, body, C.cast(tri, C.c_void_p), _p(sph), None),
                   "xdem_sim_get_mesh")
        return tri, sph

    def wrench(self, body):
        out = np.zeros(6)
        _lib.check(self.L.xdem_sim_body_wrench(self.h, body, _p(out)), "xdem_sim_body_wrench")
        return out

    def set_body(self, body, rec, plane=None):
        rec = np.ascontiguousarray(rec, dtype=np.float64)
        _lib.check(self.L.xdem_sim_set_body(self.h, body, _p(rec), C.byref(plane) if plane is not None else None),
                   "xdem_sim_set_body")

    def set_bodies(self, bodies, recs, planes=None):
        """Several poses in one call (xdem_sim_set_bodies): recs is
        len(bodies) x 15; planes a sequence of PlaneInfo, one per entry (read
        for plane bodies), or None."""
        idx = np.ascontiguousarray(bodies, dtype=np.int32)
        recs = np.ascontiguousarray(recs, dtype=np.float64).reshape(len(idx), 15)
        pl = None
        if planes is not None:
            pl = (T.PlaneInfo * len(idx))(*planes)
        _lib.check(self.L.xdem_sim_set_bodies(self.h, len(idx), idx.ctypes.data_as(C.c_void_p), _p(recs),
                                              C.cast(pl, C.c_void_p) if pl is not None else None),
                   "xdem_sim_set_bodies")

    def wrenches(self, bodies):
        """Wrenches of several bodies from one copy (xdem_sim_body_wrenches)."""
        idx = np.ascontiguousarray(bodies, dtype=np.int32)
        out = np.zeros((len(idx), 6))
        _lib.check(self.L.xdem_sim_body_wrenches(self.h, len(idx), idx.ctypes.data_as(C.c_void_p), _p(out)),
                   "xdem_sim_body_wrenches")
        return out

    def energy(self):
        ke = C.c_double()
        nc = C.c_uint()
        _lib.check(self.L.xdem_sim_energy(self.h, C.byref(ke), C.byref(nc)), "xdem_sim_energy")
        return ke.value, nc.value

    def save_part(self, path, time=0.0):
        """Part file of the current state and pair lists (xdynamics layout)."""
        _lib.check(self.L.xdem_sim_save_part(self.h, str(path).encode(), float(time)), "xdem_sim_save_part")

    def load_part(self, path):
        """Restores state and pair lists (with history) from a part file;
        returns its time."""
        t = C.c_double()
        _lib.check(self.L.xdem_sim_load_part(self.h, str(path).encode(), C.byref(t)), "xdem_sim_load_part")
        return t.value

    def status(self):
        return self.L.xdem_sim_status(self.h)

    def set_profiling(self, on):
        self.L.xdem_sim_set_profiling(self.h, int(on))

    def set_rolling_inertia(self, per_sphere):
        """1: rolling resistance reads each sphere's own inertia (inertia[3 i]);
        0 (default): the flat entry i, as the reference kernel does."""
        _lib.check(self.L.xdem_sim_set_rolling_inertia(self.h, int(per_sphere)), "xdem_sim_set_rolling_inertia")

    def set_graph(self, on):
        """Replay the step from a captured CUDA graph (identical results)."""
        _lib.check(self.L.xdem_sim_set_graph(self.h, int(on)), "xdem_sim_set_graph")

    def set_persistent(self, on, barrier_limit_ns=0):
        """Batched list steps as one cooperative kernel launch (identical
        results); each grid barrier waits at most barrier_limit_ns on the
        GPU's timer (0: one second), past which the step stops with
        XDEM_ERR_BARRIER in the status."""
        _lib.check(self.L.xdem_sim_set_persistent(self.h, int(on), int(barrier_limit_ns)),
                   "xdem_sim_set_persistent")

    def set_tune(self, nt_pairs=128, stage=16, nt_bodies=128, occ_pairs=768, occ_bodies=512, skin_div=0):
        """Block shapes and pair search of the mixed contact stage (results do
        not depend on them)."""
        t = T.Tune(nt_pairs, stage, nt_bodies, occ_pairs, occ_bodies, skin_div, 0.0)
        _lib.check(self.L.xdem_sim_set_tune(self.h, C.byref(t)), "xdem_sim_set_tune")

    def get_tune(self):
        t = T.Tune()
        _lib.check(self.L.xdem_sim_get_tune(self.h, C.byref(t)), "xdem_sim_get_tune")
        return t.as_dict()

    def autotune(self, trial_steps=10):
        """Times every candidate shape on this scene (state restored after),
        keeps the fastest; returns (best, all candidates) as dicts."""
        best = T.Tune()
        cap = C.c_uint(64)
        allv = (T.Tune * 64)()
        _lib.check(self.L.xdem_sim_autotune(self.h, int(trial_steps), C.byref(best), allv, C.byref(cap)),
                   "xdem_sim_autotune")
        return best.as_dict(), [allv[i].as_dict() for i in range(cap.value)]

    def list_rebuilds(self):
        """Candidate-list rebuilds motion has triggered so far (mixed form)."""
        n = C.c_uint()
        _lib.check(self.L.xdem_sim_list_rebuilds(self.h, C.byref(n)), "xdem_sim_list_rebuilds")
        return n.value

    def profile(self):
        nl = C.c_uint()
        ms = C.c_double()
        nc = C.c_uint()
        self.L.xdem_sim_profile(self.h, C.byref(nl), C.byref(ms), C.byref(nc))
        return nl.value, ms.value, nc.value
