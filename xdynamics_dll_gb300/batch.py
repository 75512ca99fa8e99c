"""Batched scenes: many independent DEM scenes advanced by one handle.

`Batch(scenes)` lays the scenes out side by side on a square tiling of the
x-z plane (each translated so the scenes stay at least `gap_cells` cells
apart), concatenates their particles and planes into one scene, creates one
handle over a grid that covers the tiling and declares the scenes with
xdem_sim_set_scenes: each keeps its own particle-particle material and its
own planes, and no contact is formed between scenes.  All scenes share the
time step, gravity and contact model.  A step advances every scene; with
set_graph(True) the step is replayed from a CUDA graph, and with
set_persistent(True) a list step is one cooperative kernel launch.

This is the parameter-sweep form: a sweep over friction and restitution is
one batch whose scenes differ in their contact properties.
"""
import copy
import ctypes as C
import math

import numpy as np

from . import _lib
from . import scenes as S
from . import types as T
from .sim import Sim


def _bounds(sc):
    p = sc.pos.reshape(-1, 4)
    lo = (p[:, :3] - p[:, 3:4]).min(0)
    hi = (p[:, :3] + p[:, 3:4]).max(0)
    for pl in sc.planes:
        for f in ("xw", "w2", "w3", "w4"):
            v = getattr(pl, f)
            q = np.array([v.x, v.y, v.z])
            lo = np.minimum(lo, q)
            hi = np.maximum(hi, q)
    return lo, hi


def _shift_plane(pl, d):
    out = T.PlaneInfo()
    C.pointer(out)[0] = pl
    for f in ("xw", "w2", "w3", "w4"):
        v = getattr(out, f)
        v.x += d[0]
        v.y += d[1]
        v.z += d[2]
    return out


class Batch:
    def __init__(self, scene_list, precision=T.XDEM_MIXED, gap_cells=2):
        if not scene_list:
            raise ValueError("empty batch")
        s0 = scene_list[0]
        for sc in scene_list:
            if sc.dt != s0.dt or tuple(sc.gravity) != tuple(s0.gravity) or sc.contact_model != s0.contact_model:
                raise ValueError("the scenes of a batch share dt, gravity and contact model")
            if sc.meshes or sc.cpos is not None:
                raise ValueError("a batch holds sphere scenes with planes only")
        self.scenes = scene_list
        n = len(scene_list)
        cs = max(sc.cell_size for sc in scene_list)
        bounds = [_bounds(sc) for sc in scene_list]
        ext = np.max([hi - lo for lo, hi in bounds], axis=0)
        per_row = int(math.ceil(math.sqrt(n)))
        pitch = ext + gap_cells * cs + 2 * cs
        # whole-cell offsets: a scene's cells line up with the cells it has
        # on its own grid at origin (batch origin - offset), so it walks its
        # neighbours in the same order there and here
        offsets = []
        for k, (lo, hi) in enumerate(bounds):
            ix, iz = k % per_row, k // per_row
            d = np.array([ix * pitch[0], 0.0, iz * pitch[2]]) - np.array([lo[0], lo[1], lo[2]])
            offsets.append(np.ceil(d / cs) * cs)
        self.offsets = offsets
        # one scene over the tiling
        pos, vel, acc, ep, ev, ea, mass, inertia = [], [], [], [], [], [], [], []
        planes, plane_cp, plane_body = [], [], []
        first, plane_first = [0], [0]
        for sc, d in zip(scene_list, offsets):
            p = sc.pos.reshape(-1, 4).copy()
            p[:, :3] += d
            pos.append(p.reshape(-1))
            vel.append(sc.vel); acc.append(sc.acc); ep.append(sc.ep); ev.append(sc.ev); ea.append(sc.ea)
            mass.append(sc.mass); inertia.append(sc.inertia)
            first.append(first[-1] + sc.np_)
            for k, pl in enumerate(sc.planes):
                q = _shift_plane(pl, d)
                q.id = len(planes)
                planes.append(q)
                plane_cp.append(sc.plane_cp[k])
                rec = np.asarray(sc.plane_body[k], dtype=np.float64).copy()
                rec[1:4] += d
                plane_body.append(rec)
            plane_first.append(len(planes))
        top = max(hi[1] - lo[1] for lo, hi in bounds)
        span = np.array([per_row * pitch[0], top, int(math.ceil(n / per_row)) * pitch[2]]) + cs
        o = -1.25 * cs
        grid = tuple(S.pow2_at_least(int(math.ceil((span[i] - o) / cs)) + 2) for i in range(3))
        N = first[-1]
        comb = S.Scene(np_=N, ns=N, pos=np.concatenate(pos), vel=np.concatenate(vel), acc=np.concatenate(acc),
                       ep=np.concatenate(ep), ev=np.concatenate(ev), ea=np.concatenate(ea),
                       mass=np.concatenate(mass), inertia=np.concatenate(inertia), dt=s0.dt, cell_size=cs,
                       grid=grid, origin=(o, o, o), gravity=s0.gravity, contact_model=s0.contact_model,
                       pp_cp=s0.pp_cp, planes=planes, plane_cp=plane_cp, plane_body=plane_body,
                       name="batch", note=f"{n} scenes, {N} spheres")
        self.combined = comb
        self.first = np.asarray(first, dtype=np.uint32)
        self.plane_first = np.asarray(plane_first, dtype=np.uint32)
        self.sim = Sim(comb, precision=precision)
        cps = (T.ContactProperty * n)(*[sc.pp_cp for sc in scene_list])
        self._cps = cps
        L = self.sim.L
        _lib.check(L.xdem_sim_set_scenes(self.sim.h, n, self.first.ctypes.data_as(C.c_void_p), cps,
                                         self.plane_first.ctypes.data_as(C.c_void_p)), "xdem_sim_set_scenes")
        self.sim.nscene = n

    def scene_alone(self, k):
        """Scene k on its own, on a grid whose cells line up with its cells
        in the batch (same extents, origin shifted by its offset)."""
        sc = copy.deepcopy(self.scenes[k])
        o = np.asarray(self.combined.origin) - self.offsets[k]
        sc.origin = tuple(float(v) for v in o)
        sc.grid = self.combined.grid
        sc.cell_size = self.combined.cell_size
        return sc

    # ------------------------------------------------------------------
    def step(self, n=1):
        self.sim.step(n)

    def set_graph(self, on):
        self.sim.set_graph(on)

    def set_persistent(self, on, barrier_limit_ns=0):
        """One cooperative kernel launch per list step (see Sim.set_persistent)."""
        self.sim.set_persistent(on, barrier_limit_ns)

    def autotune(self, trial_steps=10, cache=None):
        """Block shapes for this batch from the autotuner (or from `cache`,
        a JSON file of earlier choices); see xdynamics_dll_gb300.autotune."""
        from .autotune import tune
        return tune(self.sim, trial_steps=trial_steps, cache=cache)

    def energies(self):
        """Kinetic energy and stored contacts (particle and plane) of every scene."""
        n = len(self.scenes)
        ke = np.zeros(n)
        nc = np.zeros(n, dtype=np.uint32)
        _lib.check(self.sim.L.xdem_sim_scene_energy(self.sim.h, ke.ctypes.data_as(C.c_void_p),
                                                    nc.ctypes.data_as(C.c_void_p)), "xdem_sim_scene_energy")
        return ke, nc

    def states(self):
        """Per-scene state in each scene's own coordinates."""
        st = self.sim.state()
        out = []
        for k, sc in enumerate(self.scenes):
            a, b = int(self.first[k]), int(self.first[k + 1])
            p = st["pos"].reshape(-1, 4)[a:b].copy()
            p[:, :3] -= self.offsets[k]
            out.append(dict(pos=p.reshape(-1), vel=st["vel"][3 * a:3 * b], acc=st["acc"][3 * a:3 * b],
                            ep=st["ep"][4 * a:4 * b], ev=st["ev"][4 * a:4 * b], ea=st["ea"][4 * a:4 * b]))
        return out

    def status(self):
        return self.sim.status()

    def close(self):
        self.sim.close()


def sweep(n_scenes, n_min=2000, n_max=60000, r_min=1e-3, r_max=3e-3, fric=(0.1, 0.6), rest=(0.2, 0.8),
          seed=404, dt=1e-5):
    """Scenes of the batched parameter sweep: sphere drops in a 0.1 x 0.1 m
    open box (floor and four walls), each with a particle count drawn from
    U{n_min..n_max}, radii U[r_min, r_max], and its own friction and
    restitution drawn from the given ranges; everything seeded."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_scenes):
        n = int(rng.integers(n_min, n_max + 1))
        mu = float(rng.uniform(*fric))
        e = float(rng.uniform(*rest))
        out.append(S.poly_drop(n, r_min, r_max, fric=mu, rest=e, dt=dt, seed=int(rng.integers(1 << 30))))
    return out
