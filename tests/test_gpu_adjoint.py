"""Adjoint of the FP64 trajectory (xdem_adj_* through xdynamics_dll_gb300.adjoint)
against central finite differences of the same GPU forward, against finite
differences of the CPU oracle's trajectory (the FP64 reference gradient), and
across checkpoint intervals.

Finite differences are central and Richardson-extrapolated from relative
parameter steps h = 1e-7 and h/2: the trajectory is strongly curved in the
parameters (a plain central quotient after 8 steps of the 300-sphere scene
is off by 0.19 at h = 1e-6 and 1.6e-3 at h = 1e-7, falling as h^2), and the
horizons are short enough that no contact opens, closes or changes regime
(stick/slip) within the step.
"""
import numpy as np
import pytest
import torch

from xdynamics_dll_gb300 import scenes
from xdynamics_dll_gb300 import types as T

pytestmark = pytest.mark.gpu

P0 = (0.3, 0.5, 1e7)  # friction, restitution, Young's modulus


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from xdynamics_dll_gb300 import build
    build.build()
    from xdynamics_dll_gb300 import adjoint, sim
    return adjoint, sim


def packed(n=400, seed=3):
    return scenes.random_packed(n, 1e-3, 1.5e-3, 0.05, seed, overlap=0.04, vel_scale=0.05, omega_scale=5.0)


def weights(n, seed=11):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(n, 3)), rng.normal(size=(n, 3)) * 1e-3


def lin_loss(st, w, u):
    return float((w * st["pos"].reshape(-1, 4)[:, :3]).sum() + (u * st["vel"].reshape(-1, 3)).sum())


def gpu_loss(mods, sc, nsteps, w, u, params):
    adjoint, sim = mods
    s = sim.Sim(adjoint.with_parameters(sc, *params), precision=T.XDEM_FP64)
    s.step(nsteps)
    assert s.status() == 0
    out = lin_loss(s.state(), w, u)
    s.close()
    return out


def adjoint_grads(mods, sc, nsteps, w, u, params=P0, K=10, initial=False):
    adjoint, sim = mods
    s = sim.Sim(adjoint.with_parameters(sc, *params), precision=T.XDEM_FP64)
    a = adjoint.Adjoint(s, K)
    a.forward(nsteps)
    g, x0, v0 = a.backward(w, u, initial=initial)
    a.close()
    s.close()
    return g, x0, v0


def central(f, p, i, rel=1e-7, richardson=True):
    def d(h):
        pp = list(p)
        pm = list(p)
        pp[i] += h
        pm[i] -= h
        return (f(pp) - f(pm)) / (2 * h)

    h = rel * abs(p[i])
    if not richardson:
        return d(h)
    return (4.0 * d(0.5 * h) - d(h)) / 3.0


@pytest.mark.parametrize("nsteps", [1, 25])
def test_parameter_gradients_match_central_differences(mods, nsteps):
    sc = packed()
    w, u = weights(sc.np_)
    g, _, _ = adjoint_grads(mods, sc, nsteps, w, u)
    ad = [g[:, 0].sum(), g[:, 1].sum(), (g[:, 2] + g[:, 3]).sum()]
    f = lambda p: gpu_loss(mods, sc, nsteps, w, u, p)
    for i, name in enumerate(("fric", "rest", "E")):
        fd = central(f, P0, i)
        assert abs(ad[i] - fd) <= 1e-5 * max(abs(fd), 1e-300), (nsteps, name, ad[i], fd)


def test_per_property_gradient(mods):
    """Friction of the particle pairs alone (planes unchanged)."""
    adjoint, sim = mods
    sc = packed(seed=5)
    w, u = weights(sc.np_, seed=12)
    nsteps = 10
    g, _, _ = adjoint_grads(mods, sc, nsteps, w, u)

    def f(mu):
        s2 = adjoint.with_parameters(sc, *P0)
        s2.pp_cp.fric = mu
        s = sim.Sim(s2, precision=T.XDEM_FP64)
        s.step(nsteps)
        out = lin_loss(s.state(), w, u)
        s.close()
        return out

    fd = central(lambda p: f(p[0]), P0, 0)
    assert abs(g[0, 0] - fd) <= 1e-5 * abs(fd), (g[0, 0], fd)
    assert abs(g[1:, 0].sum()) > 0  # the planes carry their own share


def test_initial_state_gradient(mods):
    adjoint, sim = mods
    sc = packed(seed=7)
    w, u = weights(sc.np_, seed=13)
    nsteps = 15
    _, x0, v0 = adjoint_grads(mods, sc, nsteps, w, u, initial=True)
    x0 = x0.cpu().numpy()
    v0 = v0.cpu().numpy()
    # small entries are judged against the typical entry: the difference
    # quotient of a sum over all spheres carries rounding of that size
    sx, sv = 1e-2 * np.abs(x0).max(), 1e-2 * np.abs(v0).max()
    rng = np.random.default_rng(1)
    for i in rng.choice(sc.np_, 4, replace=False):
        for c in range(3):
            def f(dx, which):
                s2 = adjoint.with_parameters(sc, *P0)
                if which == "pos":
                    s2.pos = s2.pos.copy()
                    s2.pos[4 * i + c] += dx
                else:
                    s2.vel = s2.vel.copy()
                    s2.vel[3 * i + c] += dx
                s = sim.Sim(s2, precision=T.XDEM_FP64)
                s.step(nsteps)
                out = lin_loss(s.state(), w, u)
                s.close()
                return out

            hx = 1e-10
            fd = (f(hx, "pos") - f(-hx, "pos")) / (2 * hx)
            assert abs(x0[i, c] - fd) <= 1e-4 * max(abs(fd), sx), (i, c, x0[i, c], fd)
            hv = 1e-8
            fd = (f(hv, "vel") - f(-hv, "vel")) / (2 * hv)
            assert abs(v0[i, c] - fd) <= 1e-4 * max(abs(fd), sv), (i, c, v0[i, c], fd)


def test_checkpoint_interval_does_not_change_the_gradient(mods):
    sc = packed(seed=9)
    w, u = weights(sc.np_, seed=14)
    ref = None
    for K in (1, 4, 23, 100):
        g, x0, _ = adjoint_grads(mods, sc, 23, w, u, K=K, initial=True)
        cur = (g, x0.cpu().numpy())
        if ref is None:
            ref = cur
        else:
            assert np.array_equal(ref[0], cur[0]), K
            assert np.array_equal(ref[1], cur[1]), K


def test_gradient_matches_oracle_finite_differences(mods, oracle):
    """The FP64 reference gradient: central differences of the CPU oracle's
    own trajectory (the restated reference step)."""
    import kseq
    adjoint, _ = mods
    sc = packed(n=300, seed=15)
    w, u = weights(sc.np_, seed=16)
    nsteps = 8
    g, _, _ = adjoint_grads(mods, sc, nsteps, w, u)
    ad = [g[:, 0].sum(), g[:, 1].sum(), (g[:, 2] + g[:, 3]).sum()]
    be = kseq.OracleBackend(oracle)

    def f(p):
        s2 = adjoint.with_parameters(sc, *p)
        s = kseq.state_arrays(s2)
        for _ in range(nsteps):
            _, st, _ = kseq.sphere_step(be, s2, s, compat=0)
            assert st == 0
        return float((w * s["pos"].reshape(-1, 4)[:, :3]).sum() + (u * s["vel"].reshape(-1, 3)).sum())

    for i, name in enumerate(("fric", "rest", "E")):
        fd = central(f, P0, i)
        assert abs(ad[i] - fd) <= 1e-5 * abs(fd), (name, ad[i], fd)


def test_column_collapse_calibration_gradient(mods):
    """The calibration loss (MSE of the radial height profile against the
    profile of hidden parameters 0.35 / 0.45) through the autograd.Function,
    against central differences of the same loss."""
    adjoint, _ = mods
    sc = scenes.column_collapse(n_target=3000, R=0.03, H=0.05, v0=0.5, seed=77)
    nsteps, K = 300, 100
    center, r_max = (0.0, 0.0), 0.04
    dev = torch.device("cuda")

    def profile(p, grad=False):
        t = [torch.tensor(v, dtype=torch.float64, device=dev, requires_grad=grad) for v in p]
        pos = adjoint.trajectory(t[0], t[1], t[2], sc, nsteps, K)
        return adjoint.radial_height_profile(pos, center, r_max), t

    target, _ = profile((0.35, 0.45, 1e7))
    target = target.detach()
    prof, t = profile(P0, grad=True)
    loss = ((prof - target) ** 2).mean()
    loss.backward()
    ad = [float(x.grad) for x in t]

    def f(p):
        pr, _ = profile(p)
        return float(((pr - target) ** 2).mean())

    for i, name in enumerate(("fric", "rest", "E")):
        fd = central(f, P0, i, rel=1e-5, richardson=False)
        assert abs(ad[i] - fd) <= 1e-3 * max(abs(fd), 1e-300), (name, ad[i], fd)


def test_full_calibration_scene_gradient(mods):
    """The full calibration scene (66,099 spheres of radius 1.5 mm in a
    0.1 x 0.3 m column) over 2,600 steps with checkpoints every 100: the
    adjoint against central differences of the same loss.  Over this horizon
    the layers fall and the lowest ones bounce off the floor with vertical
    motion only, so friction has exactly zero influence on both sides and the
    loss is smooth in restitution and E.  Later (about 3,000 steps on) the
    layers collide with tangential slip and the loss turns discontinuous in
    the parameters: the reference's normal damping term beta (v . n) makes
    the contact force jump when a contact opens, so a parameter change that
    moves an opening across a step boundary moves the loss by a finite
    amount, and difference quotients grow like 1/h."""
    adjoint, _ = mods
    sc = scenes.column_collapse()
    nsteps, K = 2600, 100
    center, r_max = (0.0, 0.0), 0.15
    dev = torch.device("cuda")

    def profile(p, grad=False):
        t = [torch.tensor(v, dtype=torch.float64, device=dev, requires_grad=grad) for v in p]
        pos = adjoint.trajectory(t[0], t[1], t[2], sc, nsteps, K)
        return adjoint.radial_height_profile(pos, center, r_max), t

    target, _ = profile((0.35, 0.45, 1e7))
    target = target.detach()
    prof, t = profile(P0, grad=True)
    loss = ((prof - target) ** 2).mean()
    loss.backward()
    ad = [float(x.grad) for x in t]
    assert ad[0] == 0.0 and ad[1] != 0.0 and ad[2] != 0.0

    def f(p):
        pr, _ = profile(p)
        return float(((pr - target) ** 2).mean())

    for i in (1, 2):
        fd = central(f, P0, i, rel=1e-6, richardson=False)
        assert abs(ad[i] - fd) <= 1e-3 * abs(fd), (i, ad[i], fd)


def all_property_directions(nprop):
    """Friction, restitution and E (both moduli) moved together in every
    contact property, as adjoint.with_parameters applies them: [3, nprop, 4]
    of d(fric, rest, Ei, Ej)."""
    d = np.zeros((3, nprop, 4))
    d[0, :, 0] = 1.0
    d[1, :, 1] = 1.0
    d[2, :, 2] = d[2, :, 3] = 1.0
    return d


def test_tangent_matches_adjoint_and_differences(mods):
    """Forward mode (xdem_adj_tangent) on 400 packed spheres with 5 planes
    over 25 steps: w . dx_N + u . dv_N in each parameter direction equals the
    adjoint's grad . d (the same linearisation, accumulated the other way)
    and the Richardson-extrapolated central differences of the loss."""
    adjoint, sim = mods
    sc = packed()
    w, u = weights(sc.np_)
    nsteps = 25
    s = sim.Sim(adjoint.with_parameters(sc, *P0), precision=T.XDEM_FP64)
    a = adjoint.Adjoint(s, 10)
    a.forward(nsteps)
    D = all_property_directions(a.info()[0])
    tp, tv = a.tangent(D, velocities=True)
    g, _, _ = a.backward(w, u)
    a.close()
    s.close()
    wt, ut = torch.from_numpy(w).cuda(), torch.from_numpy(u).cuda()
    jvp = [float((wt * tp[k]).sum() + (ut * tv[k]).sum()) for k in range(3)]
    vjp = [float((g * D[k]).sum()) for k in range(3)]
    for k in range(3):
        assert abs(jvp[k] - vjp[k]) <= 1e-9 * abs(vjp[k]), (k, jvp[k], vjp[k])
    f = lambda p: gpu_loss(mods, sc, nsteps, w, u, p)
    for k in range(3):
        fd = central(f, P0, k)
        assert abs(jvp[k] - fd) <= 1e-5 * abs(fd), (k, jvp[k], fd)


def calibration_derivatives(mods, nsteps, K=100):
    """Adjoint and forward-mode derivatives of a radial-profile loss of the
    full calibration scene after nsteps, in friction, restitution and E:
    (jvp[3], vjp[3], cancellation sum|dl * t| / |sum dl * t| per direction)."""
    adjoint, sim = mods
    sc = scenes.column_collapse()
    s = sim.Sim(adjoint.with_parameters(sc, *P0), precision=T.XDEM_FP64)
    a = adjoint.Adjoint(s, K)
    a.forward(nsteps)
    pos = torch.from_numpy(s.state()["pos"].reshape(-1, 4)[:, :3].copy()).cuda().requires_grad_(True)
    prof = adjoint.radial_height_profile(pos, (0.0, 0.0), 0.15)
    loss = ((prof - 0.9 * prof.detach()) ** 2).mean()
    loss.backward()
    dl = pos.grad.detach().contiguous()
    D = all_property_directions(a.info()[0])
    tp = a.tangent(D)
    g, _, _ = a.backward(dl)
    a.close()
    s.close()
    jvp = [float((dl * tp[k]).sum()) for k in range(3)]
    vjp = [float((g * D[k]).sum()) for k in range(3)]
    cancel = [float((dl * tp[k]).abs().sum()) / max(abs(jvp[k]), 1e-300) for k in range(3)]
    return jvp, vjp, cancel


def test_full_calibration_scene_tangent_equals_adjoint(mods):
    """The full calibration scene: the adjoint's gradient of a radial-profile
    loss against the forward-mode derivative along the same trajectory.
    After 3,000 steps (layers fallen and bounced, friction without
    influence) the two agree to 1e-9.  Over the configuration's 4,000 steps
    the layers slip against each other and the derivative grows by about
    1e14 in the last 1,000 steps: the reference's tangential force keeps its
    full magnitude at any slip speed, so its direction derivative goes as
    1/|slip| for slips the forward resolves to a few digits, and the two
    accumulation orders differ at 1e-5 to 1e-4 (measured 2.6e-5, 1.2e-4 with
    a 488-fold cancellation, 8.8e-6).  Friction's derivative is not zero
    there; difference quotients do not converge at all."""
    jvp, vjp, _ = calibration_derivatives(mods, 3000)
    assert jvp[0] == 0.0 and vjp[0] == 0.0
    for k in (1, 2):
        assert vjp[k] != 0.0 and abs(jvp[k] - vjp[k]) <= 1e-9 * abs(vjp[k]), (k, jvp[k], vjp[k])
    jvp, vjp, cancel = calibration_derivatives(mods, 4000)
    assert vjp[0] != 0.0, vjp
    for k in range(3):
        assert abs(jvp[k] - vjp[k]) <= 1e-3 * abs(vjp[k]), (k, jvp[k], vjp[k], cancel[k])
