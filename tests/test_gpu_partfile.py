"""Resuming from a part file: a handle saved after N steps and loaded into a
fresh handle continues exactly as the uninterrupted run (FP64, planes and a
triangle mesh, so all three pair lists carry history), the file reads back
with the host reader, and resuming without the pair lists (what the
reference's resume does) does not."""
import numpy as np
import pytest
import torch

from xdynamics_dll_gb300 import partfile
from xdynamics_dll_gb300 import types as T

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from xdynamics_dll_gb300 import build
    build.build()
    from xdynamics_dll_gb300 import scenes, sim
    return scenes, sim


def scene(scenes):
    import test_gpu_sim
    return test_gpu_sim.scene_with_mesh(n=2500, seed=33)


def states_equal(a, b):
    for k in ("pos", "vel", "acc", "ep", "ev", "ea"):
        assert np.array_equal(a[k], b[k]), k


def test_resume_continues_the_run_exactly(mods, tmp_path):
    scenes, sim = mods
    sc = scene(scenes)
    ref = sim.Sim(sc, precision=T.XDEM_FP64)
    ref.step(12)
    a = sim.Sim(sc, precision=T.XDEM_FP64)
    a.step(7)
    p = tmp_path / "part0007.bin"
    a.save_part(p, time=7 * sc.dt)
    st7 = a.state()
    pairs7 = [a.pairs(k) for k in range(3)]
    a.close()
    # the file, read on the host
    d = partfile.read(p, ("pp", "pl", "ms"))
    assert d["time"] == 7 * sc.dt and d["np"] == sc.np_
    for k in ("pos", "vel", "acc", "ep", "ev", "ea"):
        assert np.array_equal(d[k], st7[k]), k
    for i, k in enumerate(("pp", "pl", "ms")):
        assert np.array_equal(d[k + "_count"], pairs7[i][0]), k
    assert d["pp_count"].sum() > 0 and d["pl_count"].sum() > 0 and d["ms_count"].sum() > 0
    # resumed
    b = sim.Sim(sc, precision=T.XDEM_FP64)
    assert b.load_part(p) == 7 * sc.dt
    b.step(5)
    assert b.status() == 0
    states_equal(ref.state(), b.state())
    for k, cap in enumerate((12, 3, 5)):
        (c0, i0, t0), (c1, i1, t1) = ref.pairs(k), b.pairs(k)
        assert np.array_equal(c0, c1), k
        used = (np.arange(cap)[None, :] < c0[:, None]).ravel()  # slots past the count hold stale values
        assert np.array_equal(i0[used], i1[used]), k
        assert np.array_equal(t0.reshape(-1, 2)[used], t1.reshape(-1, 2)[used]), k
    # resumed without the history: the state alone
    c = sim.Sim(sc, precision=T.XDEM_FP64)
    c.set_state(d["pos"], d["vel"], d["acc"], d["ep"], d["ev"], d["ea"], sc.mass, sc.inertia)
    c.step(5)
    assert not np.array_equal(ref.state()["vel"], c.state()["vel"])
