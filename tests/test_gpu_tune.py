"""Block-shape autotuning of the mixed contact stage (xdem_sim_set_tune /
xdem_sim_autotune): every shape and pair search (stencil walk or candidate
lists) gives the same state bit for bit, tuning leaves the simulation where
it was, wrench-keeping handles refuse unequal shapes, and the cache answers
a repeated workload without measuring."""
import numpy as np
import pytest
import torch

from xdynamics_dll_gb300 import types as T

pytestmark = pytest.mark.gpu

SHAPES = [(64, 8, 64, 768, 512, 0), (128, 16, 128, 1024, 768, 16), (256, 16, 64, 768, 1024, 8),
          (256, 8, 256, 1024, 512, 32), (64, 16, 256, 768, 768, 16)]


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
        s2.set_tune(nt, 16, nt, 1024 if nt == 128 else 768, ob, 16 if nt == 64 else 0)
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
    assert not from_cache and len(best["candidates"]) == 12 + 9 + 3
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


@pytest.mark.parametrize("skin_div", [8, 32])
def test_candidate_lists_match_the_stencil_walk(mods, skin_div):
    """A moving, colliding bed over 400 steps: the lists are rebuilt many
    times (a thin skin more often) and every step matches the walk."""
    _, _, scenes, sim = mods
    sc = scenes.random_packed(3000, 1e-3, 2e-3, 0.05, 17, overlap=0.03, vel_scale=0.3, omega_scale=20.0)
    out = []
    for sd in (0, skin_div):
        s = sim.Sim(sc, precision=T.XDEM_MIXED)
        s.set_tune(128, 16, 128, 768, 512, sd)
        st = []
        for _ in range(4):
            s.step(100)
            st.append((s.state(), s.pairs(0)))
        assert s.status() == 0
        out.append(st)
        s.close()
    for (a, pa), (b, pb) in zip(*out):
        states_equal(a, b)
        for x, y in zip(pa, pb):
            assert np.array_equal(x, y)


def test_candidate_lists_with_a_moving_mesh(mods):
    """A mesh body pushed through a moving bed, re-posed every five steps:
    the lists hold the particle pairs, the spheres near the mesh search its
    triangles, each re-pose makes the next step sort the cells again, and
    the list form matches the walk bit for bit."""
    _, _, scenes, sim = mods
    sc = scenes.random_packed(3000, 0.8e-3, 1.2e-3, None, seed=21, vel_scale=0.3)
    p = sc.pos.reshape(-1, 4)
    c = p[:, :3].mean(0)
    # no sphere starts inside the mesh (it would touch more triangles than a
    # sphere's five mesh slots)
    keep = np.linalg.norm(p[:, :3] - c, axis=1) > 2.5e-3 + p[:, 3] + 2e-4
    sc.np_ = sc.ns = int(keep.sum())
    sc.pos = p[keep].ravel()
    for k, w in (("vel", 3), ("acc", 3), ("ep", 4), ("ev", 4), ("ea", 4), ("inertia", 3)):
        setattr(sc, k, getattr(sc, k).reshape(-1, w)[keep].ravel())
    sc.mass = sc.mass[keep]
    mesh = scenes.uv_sphere_mesh(2.5e-3, 6, 10)
    body = T.body_record(mass=0.05, pos=c, vel=(0.5, 0.0, 0.0), ed=(0.0, 0.0, 0.2, 0.0))
    sc.meshes = [dict(vlist_local=mesh, body=body, cp=sc.pp_cp)]
    out = []
    for sd in (0, 16):
        s = sim.Sim(sc, precision=T.XDEM_MIXED)
        s.set_tune(128, 16, 128, 768, 512, sd)
        rec = body.copy()
        touched = 0
        for _ in range(40):
            rec[1] += 0.5 * 5 * sc.dt
            s.set_body(s.bodies[-1], rec)
            s.step(5)
            touched += int(s.pairs(2)[0].sum())
        assert s.status() == 0
        assert touched > 0
        if sd:
            assert s.list_rebuilds() >= 1
        out.append((s.state(), s.pairs(0), s.pairs(2)))
        s.close()
    (a, pa, ma), (b, pb, mb) = out
    states_equal(a, b)
    for x, y in zip(pa + ma, pb + mb):
        assert np.array_equal(x, y)


def test_overflowing_candidate_list_walks(mods):
    """A 3 mm sphere ringed by 40 small ones within the skin holds more
    candidates than a list keeps: it walks the stencil, the rest use lists,
    and the state matches the walk everywhere."""
    _, _, scenes, sim = mods
    rng = np.random.default_rng(5)
    n_in, n_out = 10, 30
    pts = [np.zeros(3)]
    rad = [3e-3]
    k = np.arange(n_in + n_out) + 0.5
    th = np.arccos(1 - 2 * k / (n_in + n_out))
    ph = np.pi * (1 + 5 ** 0.5) * k
    dirs = np.stack([np.cos(ph) * np.sin(th), np.sin(ph) * np.sin(th), np.cos(th)], 1)
    for i, d in enumerate(dirs):
        pts.append(d * (3.45e-3 if i % 4 == 0 and i // 4 < n_in else 3.7e-3))
        rad.append(0.5e-3)
    n = len(pts)
    sc = scenes.random_packed(n, 1e-3, 1e-3, 0.05, 3, nplanes=0)
    pos = np.zeros((n, 4))
    pos[:, :3] = np.array(pts) + 0.1
    pos[:, 3] = rad
    sc.pos = pos.ravel()
    m, J = scenes.sphere_mass_inertia(np.array(rad), 2500.0)
    sc.mass, sc.inertia = m, J.ravel()
    sc.vel = rng.normal(0, 0.02, n * 3)
    sc.gravity = (0.0, 0.0, 0.0)
    sc.cell_size = 6e-3
    out = []
    for sd in (0, 8):
        s = sim.Sim(sc, precision=T.XDEM_MIXED)
        s.set_tune(128, 16, 128, 768, 512, sd)
        s.step(20)
        assert s.status() == 0
        out.append((s.state(), s.pairs(0)))
        s.close()
    states_equal(out[0][0], out[1][0])
    assert out[0][1][0][0] >= 5  # the big sphere keeps its contacts
    for x, y in zip(out[0][1], out[1][1]):
        assert np.array_equal(x, y)
