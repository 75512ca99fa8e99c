"""Traces of whole runs against the CPU oracle (oracle/xdem_oracle.c, the
reference's kernels restated in C and pinned to them), at the sizes of the
configurations:

* the first configuration, the 10,000-sphere drop (41 x 41 x 6 jittered
  lattice, r 1 mm, restitution 0.5, friction 0.3, dt 1e-5 s, 2,000 steps)
  through the FP64 scene handle, kinetic energy and stored contacts compared
  every 50 steps;
* the same lattice set down on the floor, so that the 2,000 steps cover the
  impact and compaction of all six layers rather than free fall;
* the contact model of Dahl-Hertz-Sun (contact_model 0, impl:454-474)
  through the fused FP64 handle and the mixed handle;
* the mixed handle directly against the oracle.

Kinetic energy is formed the same way on both sides from the state
(translational + rotational from the Euler-parameter rates).  Tolerances are
written in each test; the measured differences are in the assertion
messages.
"""
import numpy as np
import pytest

import kseq
from xdynamics_dll_gb300 import scenes, types as T

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def simmod():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from xdynamics_dll_gb300 import build, sim
    build.build()
    return sim


def kinetic_energy(vel, ep, ev, mass, inertia):
    """0.5 m v.v + 0.5 w.J w, w = 2 L(e) e_dot the body-frame angular
    velocity (rows of impl:77-79)."""
    v = vel.reshape(-1, 3)
    e = ep.reshape(-1, 4)
    d = ev.reshape(-1, 4)
    J = inertia.reshape(-1, 3)
    w0 = 2.0 * (-e[:, 1] * d[:, 0] + e[:, 0] * d[:, 1] + e[:, 3] * d[:, 2] - e[:, 2] * d[:, 3])
    w1 = 2.0 * (-e[:, 2] * d[:, 0] - e[:, 3] * d[:, 1] + e[:, 0] * d[:, 2] + e[:, 1] * d[:, 3])
    w2 = 2.0 * (-e[:, 3] * d[:, 0] + e[:, 2] * d[:, 1] - e[:, 1] * d[:, 2] + e[:, 0] * d[:, 3])
    return float(0.5 * (mass * (v * v).sum(1)).sum() + 0.5 * (J[:, 0] * w0 ** 2 + J[:, 1] * w1 ** 2 +
                                                             J[:, 2] * w2 ** 2).sum())


def trace(simmod, oracle, sc, steps, every, precision=T.XDEM_FP64):
    """Runs the handle and the oracle side by side; returns per sample
    (KE handle, KE oracle, contacts handle, contacts oracle)."""
    sm = simmod.Sim(sc, precision=precision)
    s = kseq.state_arrays(sc)
    be = kseq.OracleBackend(oracle)
    out = []
    for k in range(steps):
        sm.step(1)
        kseq.sphere_step(be, sc, s, (), compat=0)
        if (k + 1) % every == 0:
            st = sm.state()
            cg = int(sm.pairs(0)[0].sum() + sm.pairs(1)[0].sum())
            co = int(s["pp_count"].sum() + s["pl_count"].sum())
            out.append((kinetic_energy(st["vel"], st["ep"], st["ev"], sc.mass, sc.inertia),
                        kinetic_energy(s["vel"], s["ep"], s["ev"], sc.mass, sc.inertia), cg, co))
    assert sm.status() == 0
    sm.close()
    return np.array(out)


def test_sphere_drop_configuration_trace(simmod, oracle):
    sc = scenes.sphere_drop()
    assert sc.np_ == 41 * 41 * 6
    tr = trace(simmod, oracle, sc, 2000, 50)
    rel = np.abs(tr[:, 0] - tr[:, 1]) / tr[:, 1]
    # free fall of the lattice: the FP64 step and the oracle differ only by
    # pow(x, 1.5) vs x*sqrt(x) and the closed-form Euler-parameter solve
    assert rel.max() < 1e-12, rel.max()
    assert np.array_equal(tr[:, 2], tr[:, 3]), (tr[:, 2], tr[:, 3])


def test_sphere_drop_impact_trace(simmod, oracle):
    """The configuration's lattice starting 0.1 mm above the floor: all six
    layers land and compact within the 2,000 steps."""
    sc = scenes.sphere_drop()
    p = sc.pos.reshape(-1, 4)
    p[:, 1] -= p[:, 1].min() - p[:, 3] - 1e-4
    tr = trace(simmod, oracle, sc, 2000, 50)
    assert tr[-1, 3] > sc.np_  # more than one stored contact per sphere by the end
    rel = np.abs(tr[:, 0] - tr[:, 1]) / tr[:, 1]
    dc = np.abs(tr[:, 2] - tr[:, 3])
    # identical until the layers collide; from then on repeated collisions
    # amplify the last-bit differences (pow(x, 1.5) vs x*sqrt(x), the
    # closed-form Euler-parameter solve) as they would amplify any change of
    # summation order, and the kinetic energy being dissipated makes the
    # relative difference grow further (measured 4.2e-5 at step 2,000)
    assert rel[:10].max() < 1e-12, rel[:10]
    assert rel.max() < 1e-4, (rel.max(), dc.max())
    assert np.all(dc <= np.maximum(2, 1e-3 * tr[:, 3])), dc.max()


@pytest.mark.parametrize("sratio", [0.0, 0.5])
@pytest.mark.parametrize("precision", [T.XDEM_FP64, T.XDEM_MIXED])
def test_dhs_contact_model_against_oracle(simmod, oracle, precision, sratio):
    """contact_model 0 (DHSModel, impl:454-474: linear tangential spring
    ks = kn sratio, damping vn sratio) on a dense random bed with planes,
    without and with the tangential spring: the fused FP64 step matches the
    oracle's state to 5e-11 of its scale over six steps with exact pair
    lists; the mixed step's contact and Euler accelerations match to 1e-4 of
    the largest, with exact pair lists after one step."""
    sc = scenes.random_packed(3000, 0.8e-3, 1.2e-3, None, seed=31)
    sc.contact_model = 0
    for cp in [sc.pp_cp] + list(sc.plane_cp):
        cp.sratio = sratio
    sm = simmod.Sim(sc, precision=precision)
    s = kseq.state_arrays(sc)
    be = kseq.OracleBackend(oracle)
    steps = 6 if precision == T.XDEM_FP64 else 1
    for step in range(steps):
        sm.step(1)
        kseq.sphere_step(be, sc, s, (), compat=0)
        st = sm.state()
        if precision == T.XDEM_FP64:
            for k in ("pos", "vel", "acc", "ep", "ev", "ea"):
                scale = max(np.abs(s[k]).max(), 1e-300)
                # without a tangential spring no contact turns a sphere and
                # the Euler accelerations are the gyroscopic terms alone,
                # where the closed-form solve and the reference's 4 x 4
                # solve round apart (measured 6e-11 of the scale at step 3)
                tol = 5e-10 if (k == "ea" and sratio == 0.0) else 5e-11
                assert np.abs(st[k] - s[k]).max() <= tol * scale, (step, k)
        else:
            g = np.tile(np.array(sc.gravity), sc.np_)
            fa, fb = s["acc"] - g, st["acc"] - g
            err = np.abs(fa - fb).max() / np.abs(fa).max()
            assert err < 1e-4, err
            ea_err = np.abs(s["ea"] - st["ea"]).max() / np.abs(s["ea"]).max()
            assert ea_err < 1e-4, ea_err
        for kind, (ck, ik, cap) in enumerate([("pp_count", "pp_id", 12), ("pl_count", "pl_id", 3)]):
            cnt, ids, _ = sm.pairs(kind)
            assert kseq.pairs_equal(cnt, ids, s[ck], s[ik], cap) == sc.np_, (step, ck)
    assert s["pp_count"].sum() > sc.np_ // 2 and s["pl_count"].sum() > 0
    assert sm.status() == 0


@pytest.mark.parametrize("model", [1, 0])
def test_mixed_handle_against_oracle(simmod, oracle, model):
    """The mixed step against the FP64 oracle directly, on the same input:
    one step's contact accelerations (force / mass), angular accelerations
    and the pair lists; then a 200-step kinetic-energy trace of a settling
    drop within 1e-3."""
    sc = scenes.random_packed(4000, 0.8e-3, 1.2e-3, None, seed=41 + model)
    sc.contact_model = model
    sm = simmod.Sim(sc, precision=T.XDEM_MIXED)
    s = kseq.state_arrays(sc)
    sm.step(1)
    kseq.sphere_step(kseq.OracleBackend(oracle), sc, s, (), compat=0)
    st = sm.state()
    g = np.tile(np.array(sc.gravity), sc.np_)
    fa, fb = s["acc"] - g, st["acc"] - g
    err = np.abs(fa - fb).max() / np.abs(fa).max()
    assert err < 1e-4, err
    ea_err = np.abs(s["ea"] - st["ea"]).max() / np.abs(s["ea"]).max()
    assert ea_err < 1e-4, ea_err
    for kind, (ck, ik, cap) in enumerate([("pp_count", "pp_id", 12), ("pl_count", "pl_id", 3)]):
        cnt, ids, _ = sm.pairs(kind)
        assert kseq.pairs_equal(cnt, ids, s[ck], s[ik], cap) == sc.np_, ck
    sm.close()
    drop = scenes.sphere_drop(n_per_layer_side=12, layers=4)
    p = drop.pos.reshape(-1, 4)
    p[:, 1] -= p[:, 1].min() - p[:, 3] - 1e-4
    drop.contact_model = model
    tr = trace(simmod, oracle, drop, 200, 20, precision=T.XDEM_MIXED)
    rel = np.abs(tr[:, 0] - tr[:, 1]) / tr[:, 1]
    assert rel.max() < 1e-3, rel.max()
