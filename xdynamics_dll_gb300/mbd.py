"""Host multibody side of the DEM coupling (xdem_mbd_* of include/xdem_c.h):
rigid bodies in Euler-parameter coordinates advanced by HHT-alpha, as
xIntegratorHHT (source/xdynamics_simulation/xIntegratorHHT.cpp:51-183), with
the DEM wrench entering each body's force vector.

`Multibody` wraps one system; `wheel_rig` builds the wheel testbed's drive:
a carriage sliding vertically on the ground (translational joint), the wheel
on a revolute joint to the carriage about the wheel axis, its spin driven
at a set rate.
"""
import ctypes as C

import numpy as np

from . import _lib


class _Args:
    """Float64 arrays of a call's arguments, alive until the call returns
    (a pointer to a temporary array would dangle)."""

    def __init__(self):
        self.keep = []

    def __call__(self, a):
        if a is None:
            return None
        arr = np.ascontiguousarray(a, dtype=np.float64)
        self.keep.append(arr)
        return C.c_void_p(arr.ctypes.data)


class Multibody:
    def __init__(self, dt, alpha=-0.3, gravity=(0.0, -9.80665, 0.0)):
        self.L = _lib.lib()
        h = C.c_void_p()
        _p = _Args()
        _lib.check(self.L.xdem_mbd_create(float(dt), float(alpha), _p(gravity), C.byref(h)), "xdem_mbd_create")
        self.h = h

    def close(self):
        if self.h:
            self.L.xdem_mbd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tolerance(self, eps):
        _lib.check(self.L.xdem_mbd_set_tolerance(self.h, float(eps)), "xdem_mbd_set_tolerance")

    def add_body(self, mass, inertia, pos, ep=(1.0, 0.0, 0.0, 0.0), vel=None, ed=None):
        _p = _Args()
        b = C.c_int()
        _lib.check(self.L.xdem_mbd_add_body(self.h, float(mass), _p(inertia), _p(pos), _p(ep), _p(vel), _p(ed),
                                            C.byref(b)), "xdem_mbd_add_body")
        return b.value

    def add_revolute(self, i, j, loc, axis):
        _p = _Args()
        k = C.c_int()
        _lib.check(self.L.xdem_mbd_add_revolute(self.h, i, j, _p(loc), _p(axis), C.byref(k)), "xdem_mbd_add_revolute")
        return k.value

    def add_translational(self, i, j, loc, axis):
        _p = _Args()
        k = C.c_int()
        _lib.check(self.L.xdem_mbd_add_translational(self.h, i, j, _p(loc), _p(axis), C.byref(k)),
                   "xdem_mbd_add_translational")
        return k.value

    def add_rotation_driver(self, joint, omega):
        _lib.check(self.L.xdem_mbd_add_rotation_driver(self.h, joint, float(omega)), "xdem_mbd_add_rotation_driver")

    def initialize(self):
        _lib.check(self.L.xdem_mbd_initialize(self.h), "xdem_mbd_initialize")

    def set_contact_wrench(self, body, w6):
        _p = _Args()
        _lib.check(self.L.xdem_mbd_set_contact_wrench(self.h, body, _p(w6)), "xdem_mbd_set_contact_wrench")

    def step(self):
        it = C.c_int()
        _lib.check(self.L.xdem_mbd_step(self.h, C.byref(it)), "xdem_mbd_step")
        return it.value

    def body(self, b):
        q, qd, qdd = np.zeros(7), np.zeros(7), np.zeros(7)
        ptr = lambda a: C.c_void_p(a.ctypes.data)
        _lib.check(self.L.xdem_mbd_get_body(self.h, b, ptr(q), ptr(qd), ptr(qdd)), "xdem_mbd_get_body")
        return q, qd, qdd

    def record(self, b):
        rec = np.zeros(15)
        _lib.check(self.L.xdem_mbd_body_record(self.h, b, C.c_void_p(rec.ctypes.data)), "xdem_mbd_body_record")
        return rec

    def info(self):
        t, it, nc = C.c_double(), C.c_int(), C.c_int()
        _lib.check(self.L.xdem_mbd_info(self.h, C.byref(t), C.byref(it), C.byref(nc)), "xdem_mbd_info")
        return t.value, it.value, nc.value

    def multipliers(self):
        _, _, nc = self.info()
        lam = np.zeros(max(nc, 1))
        _lib.check(self.L.xdem_mbd_multipliers(self.h, C.c_void_p(lam.ctypes.data), lam.size),
                   "xdem_mbd_multipliers")
        return lam[:nc]


def wheel_rig(dt, wheel_record, wheel_inertia, omega, carriage_mass=10.0, carriage_inertia=(0.1, 0.1, 0.1),
              axis=(0.0, 0.0, 1.0), alpha=-0.3, gravity=(0.0, -9.80665, 0.0)):
    """The wheel testbed's drive: a carriage at the wheel centre sliding
    along y on the ground, the wheel on a revolute joint to it about `axis`
    with its spin driven at `omega` rad/s (the sign gives the direction
    about the axis).  wheel_record is the wheel's 15-double body record
    (mass, centre, Euler parameters).  Returns (Multibody, wheel body)."""
    rec = np.asarray(wheel_record, dtype=np.float64)
    m = Multibody(dt, alpha, gravity)
    c = rec[1:4]
    car = m.add_body(carriage_mass, carriage_inertia, c)
    wheel = m.add_body(rec[0], wheel_inertia, c, ep=rec[7:11])
    m.add_translational(0, car, c, (0.0, 1.0, 0.0))
    j = m.add_revolute(car, wheel, c, axis)
    m.add_rotation_driver(j, omega)
    m.initialize()
    return m, wheel
