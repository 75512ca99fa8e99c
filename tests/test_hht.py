"""The host HHT-alpha multibody integrator (xdem_mbd_*, after
xIntegratorHHT.cpp:51-183 of the reference) against closed forms and an
independent ODE solution, on the CPU (it touches no GPU).

* a compound pendulum on a revolute joint, against RK4 of
  theta'' = -m g L sin(theta) / (J + m L^2) at a step a hundred times finer;
* a wheel spun by a rotation driver about its revolute joint: the angle is
  omega t, and a moment applied through the contact wrench leaves the motion
  unchanged (the drive takes it);
* the wheel testbed's drive (carriage on a vertical slider, driven wheel on
  a revolute joint) resting on a linear spring bed given through the contact
  wrench every step, as the DEM wrench is given: the sinkage oscillates as
  y_eq + A cos(w t), w^2 = k / (m_carriage + m_wheel).
"""
import numpy as np
import pytest

from xdynamics_dll_gb300 import _lib

G = 9.80665


@pytest.fixture(scope="module")
def mbd():
    import os
    if not os.path.exists(_lib.LIB_PATH):
        from xdynamics_dll_gb300 import build
        build.build()
    from xdynamics_dll_gb300 import mbd as M
    return M


def rk4_pendulum(theta0, k, t_end, dt):
    th, om = theta0, 0.0
    f = lambda th: -k * np.sin(th)
    for _ in range(int(round(t_end / dt))):
        k1t, k1o = om, f(th)
        k2t, k2o = om + 0.5 * dt * k1o, f(th + 0.5 * dt * k1t)
        k3t, k3o = om + 0.5 * dt * k2o, f(th + 0.5 * dt * k2t)
        k4t, k4o = om + dt * k3o, f(th + dt * k3t)
        th += dt / 6 * (k1t + 2 * k2t + 2 * k3t + k4t)
        om += dt / 6 * (k1o + 2 * k2o + 2 * k3o + k4o)
    return th


def test_compound_pendulum_matches_rk4(mbd):
    m, L, J, theta0, dt = 2.0, 0.5, 0.01, 0.6, 1e-3
    sys = mbd.Multibody(dt)
    sys.set_tolerance(1e-9)
    # the body hangs from the origin at angle theta0, rotated with it
    pos = (L * np.sin(theta0), -L * np.cos(theta0), 0.0)
    ep = (np.cos(0.5 * theta0), 0.0, 0.0, np.sin(0.5 * theta0))
    b = sys.add_body(m, (J, J, J), pos, ep)
    sys.add_revolute(0, b, (0.0, 0.0, 0.0), (0.0, 0.0, 1.0))
    sys.initialize()
    k = m * G * L / (J + m * L * L)
    t_end = 1.5
    for _ in range(int(round(t_end / dt))):
        sys.step()
    q, _, _ = sys.body(b)
    th = np.arctan2(q[0], -q[1])
    ref = rk4_pendulum(theta0, k, t_end, dt / 100)
    assert abs(th - ref) < 2e-4, (th, ref)
    # the body turned with the pendulum: its orientation angle equals theta
    assert abs(2.0 * np.arctan2(q[6], q[3]) - th) < 1e-8
    # on the joint: the centre stays L from the pivot, p stays unit
    assert abs(np.hypot(q[0], q[1]) - L) < 1e-10 and abs(np.dot(q[3:], q[3:]) - 1.0) < 1e-12


def test_driven_spin_follows_the_driver_and_takes_a_moment(mbd):
    dt, omega = 1e-3, -2.0
    sys = mbd.Multibody(dt)  # the reference's Newton tolerance, 1e-5
    b = sys.add_body(20.0, (0.1, 0.1, 0.2), (0.3, 0.2, 0.1))
    j = sys.add_revolute(0, b, (0.3, 0.2, 0.1), (0.0, 0.0, 1.0))
    sys.add_rotation_driver(j, omega)
    sys.initialize()
    # a moment about the axis from the bed: the drive holds the rate
    sys.set_contact_wrench(b, (0.0, 0.0, 0.0, 0.0, 0.0, 0.7))
    n = 1000
    for _ in range(n):
        sys.step()
    q, qd, _ = sys.body(b)
    th = 2.0 * np.arctan2(q[6], q[3])
    assert abs(th - omega * n * dt) < 1e-8, th
    assert np.allclose(q[:3], (0.3, 0.2, 0.1), atol=1e-12)
    # spin about z from the rates, w = 2 E(p) p_dot: the velocity-level
    # error of the position-level (index-3) constraints is O(1e-7)
    e0, e1, e2, e3 = q[3:]
    w_z = 2.0 * (-e3 * qd[3] - e2 * qd[4] + e1 * qd[5] + e0 * qd[6])
    assert abs(w_z - omega) < 1e-6, w_z
    rec = sys.record(b)
    assert rec[0] == 20.0 and np.allclose(rec[1:4], q[:3]) and np.allclose(rec[7:11], q[3:])


def test_wheel_rig_on_a_spring_bed_oscillates_as_predicted(mbd):
    """The carriage and wheel (m = 30 kg) settle on a spring bed of
    stiffness k given through the contact wrench, computed each step from
    the last step's pose (the staggered exchange of the DEM coupling):
    period 2 pi sqrt(m / k) and equilibrium y0 - m g / k.  The one-step lag
    acts as a negative damper k dt, so the amplitude grows by at most
    exp(k dt T / 2m) a period; HHT-alpha's own damping takes part of that
    back."""
    dt, k = 1e-4, 2.0e5
    m_w, m_c = 20.0, 10.0
    y0 = 0.3
    rec = np.zeros(15)
    rec[0] = m_w
    rec[1:4] = (0.5, y0, 0.15)
    rec[7] = 1.0
    sys, wheel = mbd.wheel_rig(dt, rec, (0.1, 0.1, 0.2), -2.0, carriage_mass=m_c)
    M = m_w + m_c
    y_eq = y0 - M * G / k
    w = np.sqrt(k / M)
    T = 2.0 * np.pi / w
    ys = []
    for _ in range(6000):
        q, _, _ = sys.body(wheel)
        sys.set_contact_wrench(wheel, (0.0, k * (y0 - q[1]), 0.0, 0.0, 0.0, 0.0))
        sys.step()
        ys.append(sys.body(wheel)[0][1])
    d = np.array(ys) - y_eq
    t = dt * np.arange(1, d.size + 1)
    up = np.where((d[:-1] < 0) & (d[1:] >= 0))[0]
    tz = t[up] - d[up] * dt / (d[up + 1] - d[up])
    assert abs(np.diff(tz).mean() / T - 1.0) < 1e-4
    A0 = y0 - y_eq
    assert abs(d[up[0]:up[-1]].mean()) < 1e-2 * A0
    amps = np.array([0.5 * (d[a:b].max() - d[a:b].min()) for a, b in zip(up[:-1], up[1:])])
    growth = np.mean(amps[1:] / amps[:-1])
    assert 1.0 < growth < np.exp(k * dt * T / (2.0 * M)), growth
    q, _, _ = sys.body(wheel)
    assert abs(q[0] - 0.5) < 1e-12 and abs(q[2] - 0.15) < 1e-12
    assert abs(2.0 * np.arctan2(q[6], q[3]) - (-2.0 * t[-1])) < 1e-7
    _, it, nc = sys.info()
    assert nc == 5 + 5 + 1 + 2 and 1 <= it <= 10


def test_argument_checks(mbd):
    L = _lib.lib()
    import ctypes as C
    h = C.c_void_p()
    assert L.xdem_mbd_create(0.0, -0.3, None, C.byref(h)) != 0
    assert L.xdem_mbd_create(1e-3, -0.5, None, C.byref(h)) != 0  # alpha outside [-1/3, 0]
    sys = mbd.Multibody(1e-3)
    with pytest.raises(_lib.XdemError):
        sys.step()  # not initialised
    with pytest.raises(_lib.XdemError):
        sys.add_body(-1.0, (1, 1, 1), (0, 0, 0))
    b = sys.add_body(1.0, (1, 1, 1), (0, 0, 0))
    with pytest.raises(_lib.XdemError):
        sys.add_revolute(0, 5, (0, 0, 0), (0, 0, 1))
    with pytest.raises(_lib.XdemError):
        sys.add_revolute(0, b, (0, 0, 0), (0, 0, 0))


def test_failed_step_leaves_the_system_as_it_was(mbd):
    """A Newton loop that cannot meet its tolerance (1e-300 sits below the
    residual's rounding) fails after 100 iterations; the bodies, the time
    and the multipliers stay at the last completed step, and the system
    steps on once the tolerance is reachable again."""
    dt = 1e-3
    sys = mbd.Multibody(dt)
    b = sys.add_body(2.0, (0.01, 0.01, 0.01), (0.3, -0.4, 0.0))
    sys.add_revolute(0, b, (0.0, 0.0, 0.0), (0.0, 0.0, 1.0))
    sys.initialize()
    for _ in range(5):
        sys.step()
    before = [a.copy() for a in sys.body(b)]
    t0, _, _ = sys.info()
    lam0 = sys.multipliers().copy()
    sys.set_tolerance(1e-300)
    with pytest.raises(_lib.XdemError):
        sys.step()
    after = sys.body(b)
    assert all(np.array_equal(x, y) for x, y in zip(before, after))
    t1, _, _ = sys.info()
    assert t1 == t0 and np.array_equal(sys.multipliers(), lam0)
    sys.set_tolerance(1e-5)
    sys.step()
    assert sys.info()[0] == pytest.approx(t0 + dt)
