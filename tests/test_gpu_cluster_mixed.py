"""Mixed-precision cluster step (FP32 contact geometry and forces, FP64
state) against the FP64 cluster step of the same handle API, which
tests/test_gpu_sim.py pins to the CPU oracle bit for bit.

Reference kernels: impl:149-190 (cluster position), 224-287 (cluster
velocity), 485-611 (member pairs, |id - k| <= neach skipped), 817-948
(cluster-plane contact), 2111-2268 (cluster-mesh contact).
"""
import ctypes as C

import numpy as np
import pytest
import torch

import kseq
from xdynamics_dll_gb300 import scenes
from xdynamics_dll_gb300 import types as T
from xdynamics_dll_gb300._lib import XdemError

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def simmod():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from xdynamics_dll_gb300 import build
    build.build()
    from xdynamics_dll_gb300 import sim
    return sim


def bed(n=3000, seed=7, **kw):
    """Clumps of three spheres packed close (some overlap at t = 0) with
    random velocities of 1 m/s, in a trough of five planes: within a few
    hundred steps clumps collide with each other and with the planes."""
    return scenes.cluster_bed(n, spacing_factor=0.9, vel_scale=1.0, seed=seed, trough=(0.3, 0.3, 0.1), **kw)


def developed(simmod, sc, steps):
    """The scene after `steps` FP64 steps, with its pair lists (so that the
    compared step has contacts of every age and tangential history)."""
    s = simmod.Sim(sc, precision=T.XDEM_FP64)
    s.step(steps)
    assert s.status() == 0
    st = s.state()
    pairs = [s.pairs(k) for k in (0, 1)]
    s.close()
    sc2 = sc.copy()
    for k in ("pos", "vel", "acc", "ep", "ev", "ea", "cpos"):
        setattr(sc2, k, st[k].copy())
    return sc2, pairs


def start(simmod, sc, pairs, precision):
    s = simmod.Sim(sc, precision=precision)
    for k, (cnt, ids, tsd) in zip((0, 1), pairs):
        s.set_pairs(k, cnt, ids, tsd)
    return s


def contact_acc(st, sc):
    g = np.asarray(sc.gravity, dtype=np.float64)
    return st["acc"].reshape(-1, 3) - g


def test_mixed_cluster_step_matches_fp64(simmod):
    sc0 = bed()
    sc, pairs = developed(simmod, sc0, 200)
    res = {}
    for prec in (T.XDEM_FP64, T.XDEM_MIXED):
        s = start(simmod, sc, pairs, prec)
        s.step(1)
        assert s.status() == 0
        res[prec] = (s.state(), [s.pairs(k) for k in (0, 1)], [s.wrench(b) for b in s.bodies])
        s.close()
    (s64, p64, w64), (smx, pmx, wmx) = res[T.XDEM_FP64], res[T.XDEM_MIXED]
    # the same contacts, in the same slots
    assert kseq.pairs_equal(pmx[0][0], pmx[0][1], p64[0][0], p64[0][1], 12) == sc.np_
    assert kseq.pairs_equal(pmx[1][0], pmx[1][1], p64[1][0], p64[1][1], 3) == sc.np_
    assert p64[0][0].sum() > 200 and p64[1][0].sum() > 20  # contacts to compare
    # contact accelerations (linear and Euler-parameter) to 1e-4 of the largest
    a64, amx = contact_acc(s64, sc), contact_acc(smx, sc)
    assert np.abs(amx - a64).max() <= 1e-4 * np.abs(a64).max()
    assert np.abs(smx["ea"] - s64["ea"]).max() <= 1e-4 * np.abs(s64["ea"]).max()
    # the step's positions come from the previous step's state: FP64 rounding apart
    for k in ("pos", "cpos", "ep"):
        assert np.abs(smx[k] - s64[k]).max() <= 1e-12 * np.abs(s64[k]).max(), k
    # plane wrenches
    for b, (x, y) in enumerate(zip(w64, wmx)):
        if np.abs(x).max() == 0.0:
            assert np.abs(y).max() == 0.0, b
            continue
        assert np.abs(y - x).max() <= 1e-4 * np.abs(x).max(), (b, x, y)


def test_mixed_cluster_members_stay_on_their_cluster(simmod):
    """After many steps every member centre is x_c + A(e) rloc of its
    cluster's FP64 state to ~1e-15 m."""
    sc = bed(n=1500, seed=3)
    s = simmod.Sim(sc, precision=T.XDEM_MIXED)
    s.step(300)
    assert s.status() == 0
    st = s.state()
    s.close()
    e = st["ep"].reshape(-1, 4)
    e0, e1, e2, e3 = e.T
    A = np.empty((sc.ns, 3, 3))
    A[:, 0] = np.stack([2 * (e0 * e0 + e1 * e1 - 0.5), 2 * (e1 * e2 - e0 * e3), 2 * (e1 * e3 + e0 * e2)], 1)
    A[:, 1] = np.stack([2 * (e1 * e2 + e0 * e3), 2 * (e0 * e0 + e2 * e2 - 0.5), 2 * (e2 * e3 - e0 * e1)], 1)
    A[:, 2] = np.stack([2 * (e1 * e3 - e0 * e2), 2 * (e2 * e3 + e0 * e1), 2 * (e0 * e0 + e3 * e3 - 0.5)], 1)
    rloc = sc.rloc.reshape(-1, 3)
    want = st["cpos"].reshape(-1, 4)[:, None, :3] + np.einsum("nij,kj->nki", A, rloc)
    got = st["pos"].reshape(sc.ns, -1, 4)[:, :, :3]
    assert np.abs(got - want).max() < 1e-14
    # the Euler parameters take FP32 increments, renormalised each step to
    # second order from the FP64 norm: |e| stays within the FP32 rounding of
    # one step's increment (|de| 2^-24, de ~ dt |e_dot|), which the next
    # step's renormalisation removes again
    assert np.abs(np.linalg.norm(e, axis=1) - 1.0).max() < 1e-9


def test_mixed_cluster_energy_follows_fp64(simmod):
    """Kinetic energy of the colliding bed, mixed against FP64, over 400
    steps: within 1e-3 relative at every sample."""
    sc = bed(n=2000, seed=11)
    a = simmod.Sim(sc, precision=T.XDEM_FP64)
    b = simmod.Sim(sc, precision=T.XDEM_MIXED)
    worst = 0.0
    for _ in range(20):
        a.step(20)
        b.step(20)
        ka, _ = a.energy()
        kb, _ = b.energy()
        worst = max(worst, abs(ka - kb) / max(ka, 1e-30))
    assert a.status() == 0 and b.status() == 0
    a.close()
    b.close()
    assert worst < 1e-3, worst


def test_mixed_cluster_lists_match_walk(simmod):
    """Candidate lists visit the contacts in the stencil walk's order, so the
    list and walk forms of the cluster step agree bit for bit; graph replay
    agrees with eager steps."""
    sc = bed(n=2000, seed=5)
    out = []
    for skin, graph in ((0, False), (16, False), (16, True)):
        s = simmod.Sim(sc, precision=T.XDEM_MIXED)
        s.set_tune(skin_div=skin)
        s.set_graph(graph)
        s.step(150)
        assert s.status() == 0
        out.append((s.state(), s.pairs(0)))
        if skin:
            assert s.list_rebuilds() >= 1
        s.close()
    for st, pr in out[1:]:
        for k in ("pos", "vel", "ep", "ev", "cpos"):
            assert np.array_equal(st[k], out[0][0][k]), k
        for x, y in zip(pr, out[0][1]):
            assert np.array_equal(x, y)


def test_mixed_cluster_mesh_matches_fp64(simmod):
    """The reference's cluster bed with its triangle mesh (the launcher
    fixture): one step of both forms from the same state."""
    sc, _, meshes, _ = kseq.load_ref_fixture("cluster")
    sc.meshes = [dict(vlist_local=meshes[0]["vlist"], body=meshes[0]["body"], cp=meshes[0]["cp"])]
    res = {}
    for prec in (T.XDEM_FP64, T.XDEM_MIXED):
        s = simmod.Sim(sc, precision=prec)
        s.step(2)
        assert s.status() == 0
        res[prec] = (s.state(), s.pairs(2), [s.wrench(b) for b in s.bodies])
        s.close()
    (s64, m64, w64), (smx, mmx, wmx) = res[T.XDEM_FP64], res[T.XDEM_MIXED]
    assert m64[0].sum() > 0  # members touch the mesh
    assert kseq.pairs_equal(mmx[0], mmx[1], m64[0], m64[1], 5) == sc.np_
    a64, amx = contact_acc(s64, sc), contact_acc(smx, sc)
    assert np.abs(amx - a64).max() <= 1e-4 * np.abs(a64).max()
    for b, (x, y) in enumerate(zip(w64, wmx)):
        scale = np.abs(x).max()
        assert np.abs(y - x).max() <= 1e-4 * max(scale, 1e-30) or scale == 0.0, (b, x, y)


def test_mixed_cluster_autotune_restores_state(simmod):
    sc = bed(n=1000, seed=9)
    s = simmod.Sim(sc, precision=T.XDEM_MIXED)
    s.step(5)
    before = s.state()
    best, tried = s.autotune(trial_steps=3)
    assert len(tried) > 0
    after = s.state()
    for k in before:
        assert np.array_equal(before[k], after[k]), k
    s.step(5)
    assert s.status() == 0
    s.close()


def test_mixed_cluster_refusals(simmod):
    """What the mixed cluster step does not carry is refused at the step,
    not run in another precision: rolling resistance, cohesion, and cluster
    types with different member counts."""
    sc = bed(n=200, seed=1)
    sc.pp_cp = scenes.default_material(rfric=0.1)
    s = simmod.Sim(sc, precision=T.XDEM_MIXED)
    with pytest.raises(XdemError):
        s.step(1)
    s.close()
    sc = bed(n=200, seed=1)
    s = simmod.Sim(sc, precision=T.XDEM_MIXED)
    xci = np.array([0, 0, 100, 3, 300, 100, 100, 2], dtype=np.uint32)
    rloc = np.zeros(5 * 3)
    r = s.L.xdem_sim_set_clusters(s.h, C.c_void_p(sc.cpos.ctypes.data), C.c_void_p(xci.ctypes.data), 2,
                                  C.c_void_p(rloc.ctypes.data), 5)
    assert r == 0
    with pytest.raises(XdemError):
        s.step(1)
    s.close()
