"""The mixed form (FP32 contact geometry and forces, FP64 state) against the
plain FP64 form on the same scene.

First step of a small dam break, where every column rests on the floor with
an overlap of 1e-3 r_min (1e-6 m):
  * pair lists (particle-particle and particle-plane) identical;
  * contact accelerations within 1e-4 of the largest, per sphere;
  * every plane's wrench within 1e-4 relative.
Planes that are orthonormal rectangles take the float-pair local-coordinate
test; other planes (the cube form, whose corner fields hold edge vectors)
take the FP64 test inside the mixed kernel; both are checked.
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


def _cube_scene(sc):
    out = sc.copy()
    top = float(sc.pos.reshape(-1, 4)[:, 1].max()) + 0.01
    planes = T.cube_planes((0.0, 0.0, 0.0), (1.0, top, 0.4))
    out.planes = planes
    out.plane_cp = [sc.pp_cp] * len(planes)
    out.plane_body = [T.body_record() for _ in planes]
    return out


def _compare_first_step(simmod, sc):
    a = simmod.Sim(sc, precision=T.XDEM_FP64)
    b = simmod.Sim(sc, precision=T.XDEM_MIXED)
    a.step(1)
    b.step(1)
    assert a.status() == 0 and b.status() == 0
    for kind, cap in ((0, 12), (1, 3)):
        ca, ia, _ = a.pairs(kind)
        cb, ib, _ = b.pairs(kind)
        assert kseq.pairs_equal(ca, ia, cb, ib, cap) == sc.np_, kind
    sa, sb = a.state(), b.state()
    g = np.tile(np.array(sc.gravity), sc.np_)
    fa, fb = sa["acc"] - g, sb["acc"] - g
    scale = np.abs(fa).max()
    assert scale > 0
    assert np.abs(fa - fb).max() <= 1e-4 * scale
    touched = 0
    for body in range(len(sc.planes)):
        wa, wb = a.wrench(body), b.wrench(body)
        for part in (slice(0, 3), slice(3, 6)):
            s = np.abs(wa[part]).max()
            if s > 0:
                touched += 1
                assert np.abs(wa[part] - wb[part]).max() <= 1e-4 * s, (body, wa, wb)
            else:
                assert np.abs(wb[part]).max() == 0.0, (body, wb)
    assert touched >= 2  # the floor carries every column
    a.close()
    b.close()


def test_mixed_first_step_rect_planes(simmod):
    _compare_first_step(simmod, scenes.dam_break(n_target=6000))


def test_mixed_first_step_cube_planes(simmod):
    _compare_first_step(simmod, _cube_scene(scenes.dam_break(n_target=6000)))


def test_mixed_kinetic_energy_1000_steps(simmod):
    """Kinetic-energy error of the mixed form against plain FP64 over 1,000
    steps of a small dam break (the columns compress under gravity and ring):
    at most 1e-4 relative at every 10th step, contact counts equal, and the
    velocities within 1e-4 of the largest after the run.  The records of
    every later step come from the contact kernel's own tail, so this also
    checks what the first-step tests cannot: the next-step offsets."""
    sc = scenes.dam_break(n_target=6000)
    a = simmod.Sim(sc, precision=T.XDEM_FP64)
    b = simmod.Sim(sc, precision=T.XDEM_MIXED)
    worst = 0.0
    for _ in range(100):
        a.step(10)
        b.step(10)
        ka, ca = a.energy()
        kb, cb = b.energy()
        worst = max(worst, abs(ka - kb) / ka)
        assert ca == cb
    assert a.status() == 0 and b.status() == 0
    assert worst <= 1e-4, worst
    va, vb = a.state()["vel"], b.state()["vel"]
    assert np.abs(va - vb).max() <= 1e-4 * np.abs(va).max()
    a.close()
    b.close()
