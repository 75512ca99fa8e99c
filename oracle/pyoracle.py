"""ctypes bindings of the CPU oracle (test infrastructure only).

`Oracle` wraps oracle/liboracle.so (the C restatement in xdem_oracle.c);
`RefKernels` wraps oracle/_ref/libxdem_ref.so (the reference's own kernels
compiled for the host, present only where the reference sources were
available at build time).  Only the tests, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py use this module, as the checker.
"""
import ctypes as C
import os

import numpy as np

from xdynamics_dll_gb300 import types as T

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libxdem_ref.so")


def _p(a):
    """Pointer to a numpy array's data (None passes NULL)."""
    if a is None:
        return None
    if isinstance(a, (C.Array, C.Structure)):
        return C.cast(C.pointer(a), C.c_void_p)
    assert a.flags["C_CONTIGUOUS"], "arrays must be C-contiguous"
    return C.c_void_p(a.ctypes.data)


def _ref(s):
    return C.byref(s) if s is not None else None


class Oracle:
    def __init__(self, path=ORACLE_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} missing: run `make -C oracle`")
        self.lib = C.CDLL(path)
        self.lib.xo_sum.restype = C.c_double
        self.lib.xo_step.restype = C.c_uint
        self.lib.xo_num_threads.restype = C.c_int

    # ---- helpers
    def threads(self):
        return self.lib.xo_num_threads()

    def set_threads(self, n):
        self.lib.xo_set_num_threads(int(n))

    # ---- kernels (argument order of xdem_oracle.h)
    def vv_update_position(self, prm, pos, ep, vel, ev, acc, ea, np_):
        self.lib.xo_vv_update_position(C.byref(prm), _p(pos), _p(ep), _p(vel), _p(ev), _p(acc), _p(ea), C.c_uint(np_))

    def vv_update_velocity(self, prm, vel, acc, ep, ev, ea, force, moment, mass, iner, np_, vel_compat=0):
        self.lib.xo_vv_update_velocity(C.byref(prm), _p(vel), _p(acc), _p(ep), _p(ev), _p(ea), _p(force),
                                       _p(moment), _p(mass), _p(iner), C.c_uint(np_), C.c_int(vel_compat))

    def hash(self, prm, hash_, index, pos, sid, np_):
        st = C.c_uint(0)
        self.lib.xo_hash(C.byref(prm), _p(hash_), _p(index), _p(pos), C.c_uint(sid), C.c_uint(np_), C.byref(st))
        return st.value

    def reorder(self, hash_, index, cstart, cend, sorted_index, n, ncell):
        self.lib.xo_reorder_cellstart(_p(hash_), _p(index), _p(cstart), _p(cend), _p(sorted_index),
                                      C.c_uint(n), C.c_uint(ncell))

    def p2p(self, prm, pos, ep, vel, ev, force, moment, mass, tmax, rres, pc, pid, tsd, sidx, cs, ce, cp, np_):
        st = C.c_uint(0)
        self.lib.xo_p2p(C.byref(prm), _p(pos), _p(ep), _p(vel), _p(ev), _p(force), _p(moment), _p(mass),
                        _p(tmax), _p(rres), _p(pc), _p(pid), _p(tsd), _p(sidx), _p(cs), _p(ce), C.byref(cp),
                        C.c_uint(np_), C.byref(st))
        return st.value

    def plane(self, prm, plane, dbi, cp, bf, pos, ep, vel, ev, force, moment, mass, tmax, rres, pc, pid, tsd, np_):
        st = C.c_uint(0)
        self.lib.xo_plane(C.byref(prm), C.byref(plane), _p(dbi), C.byref(cp), *[_p(b) for b in bf], _p(pos),
                          _p(ep), _p(vel), _p(ev), _p(force), _p(moment), _p(mass), _p(tmax), _p(rres), _p(pc),
                          _p(pid), _p(tsd), C.c_uint(np_), C.byref(st))
        return st.value

    def mesh(self, prm, dti, dbi, bf, pos, ep, vel, ev, force, moment, mass, tmax, rres, pc, pid, tsd,
             sidx, cs, ce, cp, np_, ntri):
        st = C.c_uint(0)
        self.lib.xo_mesh(C.byref(prm), _p(dti), _p(dbi), *[_p(b) for b in bf], _p(pos), _p(ep), _p(vel), _p(ev),
                         _p(force), _p(moment), _p(mass), _p(tmax), _p(rres), _p(pc), _p(pid), _p(tsd), _p(sidx),
                         _p(cs), _p(ce), C.byref(cp), C.c_uint(np_), C.c_uint(ntri), C.byref(st))
        return st.value

    def rolling(self, prm, tmax, rres, inertia, ep, ev, moment, np_, per_sphere=0):
        self.lib.xo_rolling_ex(C.byref(prm), _p(tmax), _p(rres), _p(inertia), _p(ep), _p(ev), _p(moment),
                               C.c_uint(np_), C.c_int(per_sphere))

    def update_mesh(self, dbi, vlist, sphere, dlocal, dpi, ntri):
        self.lib.xo_update_mesh(_p(dbi), _p(vlist), _p(sphere), _p(dlocal), _p(dpi), C.c_uint(ntri))

    def clusters_p2p(self, prm, pos, cpos, ep, vel, ev, force, moment, mass, tmax, rres, pc, pid, tsd,
                     sidx, cs, ce, cp, xci, np_):
        st = C.c_uint(0)
        self.lib.xo_clusters_p2p(C.byref(prm), _p(pos), _p(cpos), _p(ep), _p(vel), _p(ev), _p(force),
                                 _p(moment), _p(mass), _p(tmax), _p(rres), _p(pc), _p(pid), _p(tsd), _p(sidx),
                                 _p(cs), _p(ce), C.byref(cp), _p(xci), C.c_uint(np_), C.byref(st))
        return st.value

    def cluster_plane(self, prm, plane, dbi, bf, pos, cpos, ep, vel, ev, force, moment, cp, mass, tmax, rres,
                      pc, pid, tsd, xci, np_):
        st = C.c_uint(0)
        self.lib.xo_cluster_plane(C.byref(prm), C.byref(plane), _p(dbi), *[_p(b) for b in bf], _p(pos),
                                  _p(cpos), _p(ep), _p(vel), _p(ev), _p(force), _p(moment), C.byref(cp), _p(mass),
                                  _p(tmax), _p(rres), _p(pc), _p(pid), _p(tsd), _p(xci), C.c_uint(np_),
                                  C.byref(st))
        return st.value

    def cluster_mesh(self, prm, dti, dbi, bf, pos, cpos, ep, vel, ev, force, moment, cp, mass, tmax, rres,
                     pc, pid, tsd, sidx, cs, ce, xci, np_, ntri):
        st = C.c_uint(0)
        self.lib.xo_cluster_mesh(C.byref(prm), _p(dti), _p(dbi), *[_p(b) for b in bf], _p(pos), _p(cpos),
                                 _p(ep), _p(vel), _p(ev), _p(force), _p(moment), C.byref(cp), _p(mass), _p(tmax),
                                 _p(rres), _p(pc), _p(pid), _p(tsd), _p(sidx), _p(cs), _p(ce), _p(xci),
                                 C.c_uint(np_), C.c_uint(ntri), C.byref(st))
        return st.value

    def cylinder(self, prm, cyl, dbi, cp, bf, pos, cpos, ep, vel, ev, force, moment, mass, tmax, rres, pc, pid,
                 tsd, xci, np_):
        """xo_cylinder: cpos None for free spheres."""
        st = C.c_uint(0)
        self.lib.xo_cylinder(C.byref(prm), C.byref(cyl), _p(dbi), C.byref(cp), *[_p(b) for b in bf], _p(pos),
                             _p(cpos), _p(ep), _p(vel), _p(ev), _p(force), _p(moment), _p(mass), _p(tmax), _p(rres),
                             _p(pc), _p(pid), _p(tsd), _p(xci), C.c_uint(np_), C.byref(st))
        return st.value

    def cluster_rolling(self, prm, tmax, rres, inertia, ep, ev, moment, xci, np_):
        self.lib.xo_cluster_rolling(C.byref(prm), _p(tmax), _p(rres), _p(inertia), _p(ep), _p(ev), _p(moment),
                                    _p(xci), C.c_uint(np_))

    def vv_cluster_position(self, prm, pos, cpos, ep, rloc, vel, acc, ev, ea, xci, ns):
        self.lib.xo_vv_cluster_position(C.byref(prm), _p(pos), _p(cpos), _p(ep), _p(rloc), _p(vel), _p(acc),
                                        _p(ev), _p(ea), _p(xci), C.c_uint(ns))

    def vv_cluster_velocity(self, prm, cpos, ep, vel, acc, ev, ea, force, moment, rloc, mass, iner, xci, ns):
        self.lib.xo_vv_cluster_velocity(C.byref(prm), _p(cpos), _p(ep), _p(vel), _p(acc), _p(ev), _p(ea),
                                        _p(force), _p(moment), _p(rloc), _p(mass), _p(iner), _p(xci),
                                        C.c_uint(ns))

    def fit_sphere(self, P, Q, R, ft=0.8):
        out = np.zeros(4)
        arr = [np.ascontiguousarray(x, dtype=np.float64) for x in (P, Q, R)]
        self.lib.xo_fit_sphere_to_triangle(_p(arr[0]), _p(arr[1]), _p(arr[2]), C.c_double(ft), _p(out))
        return out

    def sum(self, a):
        return self.lib.xo_sum(_p(a), C.c_uint(a.size))


class RefKernels:
    """The reference's own kernels, compiled for the host by `make -C oracle ref`."""

    def __init__(self, path=REF_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        assert self.lib.ref_params_size() == C.sizeof(T.DemParameters)

    def set_params(self, prm):
        self.lib.ref_set_params(C.byref(prm))

    def __getattr__(self, name):
        fn = getattr(self.lib, "ref_" + name)

        def call(*args):
            conv = []
            for a in args:
                if isinstance(a, np.ndarray):
                    conv.append(_p(a))
                elif isinstance(a, C.Structure):
                    conv.append(C.byref(a))
                elif isinstance(a, (int, np.integer)):
                    conv.append(C.c_uint(a))
                else:
                    conv.append(a)
            return fn(*conv)
        return call


def ref_available():
    return os.path.exists(REF_SO)
