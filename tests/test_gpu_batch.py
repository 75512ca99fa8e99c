"""Batched scenes (xdem_sim_set_scenes, xdynamics_dll_gb300.batch) against
the same scenes run one by one.

Each scene of a batch sits on whole-cell offsets, so on its own grid at the
matching origin it walks its neighbours in the same order: pair lists must
agree exactly and the state within FP64 rounding of the translated
coordinates.  The scenes differ in friction and restitution (a parameter
sweep), which also checks that every scene uses its own material, and a
scene's energy from xdem_sim_scene_energy must match the scene run alone.
"""
import numpy as np
import pytest

from xdynamics_dll_gb300 import scenes, types as T

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from xdynamics_dll_gb300 import batch, build, sim
    build.build()
    return batch, sim


def _members():
    out = []
    for k, (mu, e) in enumerate([(0.15, 0.7), (0.5, 0.3), (0.35, 0.5)]):
        out.append(scenes.dam_break(n_target=1200 + 300 * k, block_x=0.05, block_z=0.05, box=(0.12, 0.3, 0.1),
                                    fric=mu, rest=e, seed=100 + k))
    return out


@pytest.mark.parametrize("precision", [T.XDEM_FP64, T.XDEM_MIXED])
def test_batch_matches_scenes_alone(mods, precision):
    batch, sim = mods
    members = _members()
    b = batch.Batch(members, precision=precision)
    alone = [sim.Sim(b.scene_alone(k), precision=precision) for k in range(len(members))]
    for _ in range(3):
        b.step(10)
        for s in alone:
            s.step(10)
    assert b.status() == 0 and all(s.status() == 0 for s in alone)
    states = b.states()
    st_all = b.sim.state()
    ke_b, nc_b = b.energies()
    for k, s in enumerate(alone):
        a0, a1 = int(b.first[k]), int(b.first[k + 1])
        for kind, cap in ((0, 12), (1, 3)):
            cnt_b, id_b, _ = b.sim.pairs(kind)
            cnt_a, id_a, _ = s.pairs(kind)
            cb = cnt_b[a0:a1]
            ib = id_b.reshape(-1, cap)[a0:a1].astype(np.int64)
            if kind == 0:
                ib = ib - a0  # particle ids are batch-global
            else:
                ib = ib - int(b.plane_first[k])  # plane ids too
            mask = np.arange(cap)[None, :] < cb[:, None]
            ib[~mask] = 0
            ia = id_a.reshape(-1, cap).astype(np.int64).copy()
            ia[~(np.arange(cap)[None, :] < cnt_a[:, None])] = 0
            assert np.array_equal(cb, cnt_a), (k, kind)
            assert np.array_equal(ib, ia), (k, kind)
        # FP64: rounding of the translated coordinates only; mixed: the same,
        # seen through FP32 contact forces
        tol = 1e-9 if precision == T.XDEM_FP64 else 1e-7
        sa = s.state()
        for key in ("pos", "vel", "ep", "ev"):
            x, y = states[k][key], sa[key]
            scale = max(np.abs(y).max(), 1e-30)
            assert np.abs(x - y).max() <= tol * scale, (k, key, np.abs(x - y).max(), scale)
        ke_a, nc_a = s.energy()
        assert abs(ke_b[k] - ke_a) <= 10 * tol * ke_a, (k, ke_b[k], ke_a)
    # different materials gave different scenes
    assert len(set(np.round(ke_b / ke_b.max(), 6))) == len(members)
    b.close()
    for s in alone:
        s.close()


def test_batch_graph_replay_is_identical(mods):
    batch, _ = mods
    members = _members()
    a = batch.Batch(members, precision=T.XDEM_MIXED)
    g = batch.Batch(members, precision=T.XDEM_MIXED)
    g.set_graph(True)
    a.step(7)
    g.step(7)
    sa, sg = a.sim.state(), g.sim.state()
    for k in sa:
        assert np.array_equal(sa[k], sg[k]), k
    a.close()
    g.close()


def _list_batch(batch, members, persist=False, graph=False):
    b = batch.Batch(members, precision=T.XDEM_MIXED)
    b.sim.set_tune(nt_pairs=64, stage=16, nt_bodies=64, occ_pairs=768, occ_bodies=1024, skin_div=32)
    if persist:
        b.set_persistent(True)
    if graph:
        b.set_graph(True)
    return b


def _same(a, b):
    sa, sb = a.state(), b.state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
    for kind in range(2):
        for x, y in zip(a.pairs(kind), b.pairs(kind)):
            assert np.array_equal(x, y), kind


def test_persistent_step_matches_kernels(mods):
    """A batched list step as one cooperative launch (xdem_sim_set_persistent:
    gated sort, pair phase, body phase and flag roll behind grid barriers)
    against the same steps as separate kernels: states and pair lists bit for
    bit, eager and replayed from a graph, over steps that rebuild the
    candidate lists; one kernel per step."""
    batch, _ = mods
    members = _members()
    ref = _list_batch(batch, members)
    per = _list_batch(batch, members, persist=True)
    pg = _list_batch(batch, members, persist=True, graph=True)
    # the columns start at rest: a seeded random velocity (the same in all
    # three) makes spheres cross half the skin within tens of steps, so the
    # lists are rebuilt on motion (those steps clear the last sort's cells,
    # sort and reorder inside the kernel)
    st = ref.sim.state()
    vel = st["vel"] + np.random.default_rng(7).uniform(-0.2, 0.2, st["vel"].shape)
    for b in (ref, per, pg):
        b.sim.set_state(st["pos"], vel, st["acc"], st["ep"], st["ev"], st["ea"], b.combined.mass,
                        b.combined.inertia)
    for n in (1, 5, 20, 54, 120):
        for b in (ref, per, pg):
            b.step(n)
        _same(ref.sim, per.sim)
        _same(ref.sim, pg.sim)
    assert per.sim.list_rebuilds() == ref.sim.list_rebuilds() >= 1
    for b in (ref, per, pg):
        b.step(1)
    launches, _, _ = per.sim.profile()
    assert launches == 1
    launches_ref, _, _ = ref.sim.profile()
    assert launches_ref >= 3
    _same(ref.sim, per.sim)
    for b in (ref, per, pg):
        assert b.status() == 0
        b.close()


def test_persistent_barrier_limit_stops_the_step(mods):
    """The grid barriers wait at most the host-set limit: at 1 ns a block that
    has to wait gives up at once, the step stops with XDEM_ERR_BARRIER and the
    kernel returns (no hang).  Restored to a saved state with the default
    limit, the handle steps as one that never stopped."""
    batch, _ = mods
    members = _members()
    ref = _list_batch(batch, members, persist=True)
    b = _list_batch(batch, members, persist=True)
    ref.step(4)
    b.step(4)
    st = b.sim.state()
    prs = [b.sim.pairs(k) for k in range(2)]
    b.set_persistent(True, 1)
    b.step(1)
    assert b.status() & T.XDEM_ERR_BARRIER
    b.set_persistent(True, 0)
    mass, inertia = b.combined.mass, b.combined.inertia
    for h in (ref, b):
        h.sim.set_state(st["pos"], st["vel"], st["acc"], st["ep"], st["ev"], st["ea"], mass, inertia)
        for k, pr in enumerate(prs):
            h.sim.set_pairs(k, *pr)
        h.step(12)
    _same(ref.sim, b.sim)
    assert ref.status() == 0 and b.status() == 0
    ref.close()
    b.close()
