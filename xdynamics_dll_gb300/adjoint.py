"""Gradients of a DEM trajectory with respect to material parameters.

`Adjoint` wraps xdem_adj_* of include/xdem_c.h: a reverse-mode adjoint of
the FP64 step of a scene handle, checkpointed every K steps and recomputed
in between, written by hand in CUDA (xdynamics_dll_gb300/csrc/xdem_adjoint.cu).
`Trajectory` puts it behind a torch.autograd.Function: friction,
restitution and Young's modulus in, final sphere positions out, and
`backward` returns d loss / d (friction, restitution, E) for any loss torch
can differentiate with respect to those positions (for example
`radial_height_profile` below).

The parameters apply to every contact property of the scene: friction and
restitution of the particle-particle and particle-plane pairs, and both
Young's moduli (Ei, Ej) of every pair.
"""
import ctypes as C

import numpy as np
import torch

from . import _lib
from . import types as T
from .sim import Sim


def _dptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


class Adjoint:
    """Checkpointed adjoint of `sim` (an FP64 `Sim`)."""

    def __init__(self, sim, checkpoint_every=100):
        self.sim = sim
        self.L = sim.L
        h = C.c_void_p()
        _lib.check(self.L.xdem_adj_create(sim.h, int(checkpoint_every), C.byref(h)), "xdem_adj_create")
        self.h = h
        self.K = int(checkpoint_every)

    def close(self):
        if self.h:
            self.L.xdem_adj_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, nsteps):
        """Advances the handle `nsteps` steps keeping checkpoints."""
        _lib.check(self.L.xdem_adj_forward(self.h, int(nsteps)), "xdem_adj_forward")

    def info(self):
        nprop, nsteps, nbytes = C.c_uint(), C.c_uint(), C.c_ulonglong()
        _lib.check(self.L.xdem_adj_info(self.h, C.byref(nprop), C.byref(nsteps), C.byref(nbytes)), "xdem_adj_info")
        return nprop.value, nsteps.value, nbytes.value

    def backward(self, dl_dpos, dl_dvel=None, initial=False):
        """dl_dpos / dl_dvel: float64 tensors [np, 3] (None = 0), moved to the
        GPU.  Returns (grad [nprop, 4] of d/dfric, d/drest, d/dEi, d/dEj per
        contact property, dl_dpos0, dl_dvel0) -- the last two only with
        initial=True."""
        n = self.sim.scene.np_
        nprop = self.info()[0]
        args = []
        for t in (dl_dpos, dl_dvel):
            if t is not None:
                t = torch.as_tensor(t).detach().to(device="cuda", dtype=torch.float64).contiguous()
                if t.numel() != 3 * n:
                    raise ValueError("gradient arrays are [np, 3]")
            args.append(t)
        g = np.zeros(4 * nprop)
        out0 = [torch.empty((n, 3), dtype=torch.float64, device="cuda") for _ in range(2)] if initial else [None, None]
        _lib.check(self.L.xdem_adj_backward(self.h, _dptr(args[0]), _dptr(args[1]),
                                            C.c_void_p(g.ctypes.data), _dptr(out0[0]), _dptr(out0[1])),
                   "xdem_adj_backward")
        return g.reshape(nprop, 4), out0[0], out0[1]

    def tangent(self, dparam, velocities=False):
        """Forward-mode derivative of the final state along the stored
        trajectory (xdem_adj_tangent).  dparam: [ndir, nprop, 4] (ndir <= 3)
        of d(fric, rest, Ei, Ej) per contact property.  Returns the
        derivative of the final positions, a CUDA float64 tensor [ndir, np,
        3] (and of the velocities with velocities=True)."""
        n = self.sim.scene.np_
        d = np.ascontiguousarray(dparam, dtype=np.float64)
        if d.ndim != 3 or d.shape[1:] != (self.info()[0], 4) or not 1 <= d.shape[0] <= 3:
            raise ValueError("dparam is [ndir <= 3, nprop, 4]")
        tp = torch.empty((d.shape[0], n, 3), dtype=torch.float64, device="cuda")
        tv = torch.empty_like(tp) if velocities else None
        _lib.check(self.L.xdem_adj_tangent(self.h, d.shape[0], C.c_void_p(d.ctypes.data), _dptr(tp), _dptr(tv)),
                   "xdem_adj_tangent")
        return (tp, tv) if velocities else tp


def with_parameters(scene, fric, rest, young):
    """A copy of `scene` whose contact properties all use friction `fric`,
    restitution `rest` and Young's moduli `young`."""
    sc = scene.copy()

    def cp(c):
        d = T.ContactProperty()
        C.memmove(C.addressof(d), C.addressof(c), C.sizeof(d))
        d.fric, d.rest, d.Ei, d.Ej = float(fric), float(rest), float(young), float(young)
        return d

    sc.pp_cp = cp(scene.pp_cp)
    sc.plane_cp = [cp(c) for c in scene.plane_cp]
    return sc


class Trajectory(torch.autograd.Function):
    """positions = Trajectory.apply(fric, rest, young, scene, nsteps, K):
    final sphere centres [np, 3] (float64, CUDA) after `nsteps` FP64 steps of
    `scene` run with those parameters; differentiable in the three scalars."""

    @staticmethod
    def forward(ctx, fric, rest, young, scene, nsteps, checkpoint_every):
        sc = with_parameters(scene, fric.item(), rest.item(), young.item())
        sim = Sim(sc, precision=T.XDEM_FP64)
        adj = Adjoint(sim, checkpoint_every)
        adj.forward(nsteps)
        pos = sim.state()["pos"].reshape(-1, 4)[:, :3].copy()
        ctx.adj = adj
        ctx.sim = sim
        return torch.from_numpy(pos).to(device="cuda")

    @staticmethod
    def backward(ctx, gpos):
        g, _, _ = ctx.adj.backward(gpos)
        ctx.adj.close()
        ctx.sim.close()
        dev = gpos.device
        d_fric = torch.tensor(g[:, 0].sum(), dtype=torch.float64, device=dev)
        d_rest = torch.tensor(g[:, 1].sum(), dtype=torch.float64, device=dev)
        d_young = torch.tensor((g[:, 2] + g[:, 3]).sum(), dtype=torch.float64, device=dev)
        return d_fric, d_rest, d_young, None, None, None


def trajectory(fric, rest, young, scene, nsteps, checkpoint_every=100):
    return Trajectory.apply(fric, rest, young, scene, nsteps, checkpoint_every)


def radial_height_profile(pos, center, r_max, nbins=64, width=None):
    """Smooth radial height profile of a sphere heap: for bin centres c_b over
    [0, r_max], the Gaussian-weighted (width = bin size) mean height y of the
    spheres at horizontal distance r = |(x, z) - center| near c_b."""
    width = r_max / nbins if width is None else width
    cb = (torch.arange(nbins, dtype=pos.dtype, device=pos.device) + 0.5) * (r_max / nbins)
    r = torch.sqrt((pos[:, 0] - center[0]) ** 2 + (pos[:, 2] - center[1]) ** 2)
    w = torch.exp(-0.5 * ((r[:, None] - cb[None, :]) / width) ** 2)
    return (w * pos[:, 1:2]).sum(0) / (w.sum(0) + 1e-12)
