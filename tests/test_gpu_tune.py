"""Block-shape autotuning of the mixed contact stage (xdem_sim_set_tune /
xdem_sim_autotune): every shape gives the same state bit for bit, tuning
leaves the simulation where it was, wrench-keeping handles refuse unequal
shapes, and the cache answers a repeated workload without measuring."""
import numpy as np
import pytest
import torch

from xdynamics_dll_gb300 import types as T

pytestmark = pytest.mark.gpu

SHAPES = [(64, 8, 64, 768, 512), (128, 16, 128, 1024, 768), (256, 16, 64, 768, 1024), (256, 8, 256, 1024, 512),
          (64, 16, 256, 768, 768)]


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from xdynamics_dll_gb300 import build
    build.build()
    from xdynamics_dll_gb300 import _lib, batch, scenes, sim
    return _lib, batch, scenes, sim


def members(batch):
    return batch.sweep(4, n_min=1500, n_max=5000, seed=31)


def states_equal(a, b):
    for k in ("pos", "vel", "acc", "ep", "ev", "ea"):
        assert np.array_equal(a[k], b[k]), k


def test_every_shape_gives_the_same_state(mods):
    _, batch, _, _ = mods
    ref = None
    for shp in SHAPES:
        b = batch.Batch(members(batch))
        b.sim.set_tune(*shp)
        b.step(30)
        assert b.status() == 0
        st = b.sim.state()
        pairs = b.sim.pairs(0)
        if ref is None:
            ref = (st, pairs)
        else:
            states_equal(ref[0], st)
            for x, y in zip(ref[1], pairs):
                assert np.array_equal(x, y)
        b.close()


def test_wrench_keeping_handle_needs_equal_shapes(mods):
    _lib, _, scenes, sim = mods
    sc = scenes.sphere_drop(n_per_layer_side=20, layers=3)
    s = sim.Sim(sc, precision=T.XDEM_MIXED)
    with pytest.raises(_lib.XdemError):
        s.set_tune(64, 16, 128)
    ref = None
    for nt, ob in ((64, 512), (128, 1024), (256, 768)):
        s2 = sim.Sim(sc, precision=T.XDEM_MIXED)
        s2.set_tune(nt, 16, nt, 1024 if nt == 128 else 768, ob)
        s2.step(40)
        st, w = s2.state(), s2.wrench(0)
        if ref is None:
            ref = (st, w)
        else:
            states_equal(ref[0], st)
            # block partial sums of the floor's wrench regroup with the block size
            assert np.allclose(ref[1], w, rtol=1e-5, atol=1e-12)
        s2.close()
    s.close()


def test_autotune_leaves_the_simulation_where_it_was(mods, tmp_path):
    _, batch, _, _ = mods
    a = batch.Batch(members(batch))
    best, from_cache = a.autotune(trial_steps=5, cache=str(tmp_path / "tune.json"))
    assert not from_cache and len(best["candidates"]) == 12 + 9
    assert best["contact_ms"] == min(c["contact_ms"] for c in best["candidates"])
    a.step(20)
    b = batch.Batch(members(batch))
    b.sim.set_tune(**{k: best[k] for k in T.Tune.SHAPE})
    b.step(20)
    states_equal(a.sim.state(), b.sim.state())
    # the same workload again: from the cache, nothing measured
    c = batch.Batch(members(batch))
    again, from_cache = c.autotune(trial_steps=5, cache=str(tmp_path / "tune.json"))
    assert from_cache and {k: again[k] for k in T.Tune.SHAPE} == {k: best[k] for k in T.Tune.SHAPE}
    assert c.sim.get_tune()["nt_pairs"] == best["nt_pairs"]
