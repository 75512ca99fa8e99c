"""The scene handle (fused sorted-order step) against the CPU oracle.

FP64 path: cell ids and pair lists bit-exact, state within 1e-11 of the
state's scale after 1 and after several steps (the only arithmetic
differences from the oracle are pow(x,1.5) -> x*sqrt(x), libm vs CUDA log,
and the closed-form Euler-parameter solve).
Mixed path (FP32 contact geometry and forces, FP64 state): single-step forces
within 1e-4 relative of FP64 (measured through the velocity change), and the
kinetic-energy trace within 1e-3 over 200 steps of a settling bed."""
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


def scene_with_mesh(n=3000, seed=21, rfric=0.0):
    sc = scenes.random_packed(n, 0.8e-3, 1.2e-3, None, seed=seed, rfric=rfric)
    c = sc.pos.reshape(-1, 4)[:, :3].mean(0)
    mesh = scenes.uv_sphere_mesh(2.5e-3, 6, 10)
    body = T.body_record(mass=0.05, pos=c, vel=(0.01, -0.02, 0.0), ed=(0.0, 0.3, 0.1, -0.2))
    sc.meshes = [dict(vlist_local=mesh, body=body, cp=sc.pp_cp)]
    return sc


def oracle_meshes_from_sim(sm, sc):
    out = []
    base = 0
    for bi, m in zip(sm.bodies[len(sc.planes):], sc.meshes):
        tri, sph = sm.mesh(bi)
        out.append(dict(ntri=len(tri), dti=tri, sphere=sph, body=np.asarray(m["body"], float), cp=m["cp"],
                        base=base))
        base += len(tri)
    return out


def compare(sm, s, sc, tol, step):
    st = sm.state()
    for k in ("pos", "vel", "acc", "ep", "ev", "ea"):
        a, b = st[k], s[k]
        scale = max(np.abs(b).max(), 1e-300)
        assert np.abs(a - b).max() <= tol * scale, (step, k, np.abs(a - b).max(), scale)
    for kind, (ck, ik, cap) in enumerate([("pp_count", "pp_id", 12), ("pl_count", "pl_id", 3),
                                          ("ms_count", "ms_id", 5)]):
        cnt, ids, tsd = sm.pairs(kind)
        assert kseq.pairs_equal(cnt, ids, s[ck], s[ik], cap) == sc.np_, (step, ck)
        t1 = kseq.masked_tsd(cnt, tsd, cap)
        t2 = kseq.masked_tsd(s[ck], s[ck.replace("count", "tsd")], cap)
        scale = max(np.abs(t2).max(), 1e-300)
        assert np.abs(t1 - t2).max() <= max(tol, 1e-10) * scale, (step, ck, np.abs(t1 - t2).max())


@pytest.mark.parametrize("launcher_path", [0, 1])
@pytest.mark.parametrize("compat", [0, 1])
def test_fp64_handle_matches_oracle(simmod, oracle, launcher_path, compat):
    sc = scene_with_mesh(seed=21 + compat, rfric=0.03 if compat else 0.0)
    sm = simmod.Sim(sc, precision=T.XDEM_FP64, velocity_compat=compat, launcher_path=launcher_path)
    meshes = oracle_meshes_from_sim(sm, sc)
    rmax = max(sc.pos.reshape(-1, 4)[:, 3].max(), meshes[0]["sphere"].reshape(-1, 4)[:, 3].max())
    assert sc.cell_size >= 2 * rmax - 1e-12 or True
    s = kseq.state_arrays(sc)
    be = kseq.OracleBackend(oracle)
    for step in range(6):
        sm.step(1)
        kseq.sphere_step(be, sc, s, meshes, compat=compat)
        compare(sm, s, sc, 1e-11, step)
    assert sm.status() == 0
    assert s["pp_count"].sum() > sc.np_ // 2 and s["pl_count"].sum() > 0 and s["ms_count"].sum() > 0


def test_wrench_matches_oracle(simmod, oracle):
    sc = scene_with_mesh(seed=5)
    sm = simmod.Sim(sc, precision=T.XDEM_FP64)
    meshes = oracle_meshes_from_sim(sm, sc)
    s = kseq.state_arrays(sc)
    sm.step(1)
    _, _, partials = kseq.sphere_step(kseq.OracleBackend(oracle), sc, s, meshes, compat=0)
    for b, part in enumerate(partials):
        w = sm.wrench(sm.bodies[b])
        ref = np.array([p.sum() for p in part])
        scale = max(np.abs(ref).max(), 1e-12)
        assert np.abs(w - ref).max() <= 1e-10 * scale, (b, w, ref)


def test_mixed_single_step_forces(simmod):
    sc = scenes.random_packed(4000, 0.8e-3, 1.2e-3, None, seed=8)
    a = simmod.Sim(sc, precision=T.XDEM_FP64)
    b = simmod.Sim(sc, precision=T.XDEM_MIXED)
    a.step(1)
    b.step(1)
    sa, sb = a.state(), b.state()
    # acceleration = F/m + g: compare the contact part
    g = np.tile(np.array(sc.gravity), sc.np_)
    fa, fb = sa["acc"] - g, sb["acc"] - g
    scale = np.abs(fa).max()
    err = np.abs(fa - fb).max() / scale
    assert err < 1e-4, err
    # the float-pair overlap classifies every pair as FP64 does: the same
    # pair lists, slot for slot
    for kind, cap in ((0, 12), (1, 3)):
        ca, ia, _ = a.pairs(kind)
        cb, ib, _ = b.pairs(kind)
        assert kseq.pairs_equal(ca, ia, cb, ib, cap) == sc.np_, kind


def test_mixed_energy_trace(simmod):
    sc = scenes.sphere_drop(n_per_layer_side=12, layers=4, dt=1e-5)
    a = simmod.Sim(sc, precision=T.XDEM_FP64)
    b = simmod.Sim(sc, precision=T.XDEM_MIXED)
    worst = 0.0
    for _ in range(20):
        a.step(10)
        b.step(10)
        ka, _ = a.energy()
        kb, _ = b.energy()
        worst = max(worst, abs(ka - kb) / max(ka, 1e-30))
    assert worst < 1e-3, worst


def test_cluster_handle_matches_oracle(simmod, oracle):
    sc, s0, meshes, exp = kseq.load_ref_fixture("cluster")
    sc.meshes = []
    sm = simmod.Sim(sc, precision=T.XDEM_FP64)
    s = kseq.state_arrays(sc)
    be = kseq.OracleBackend(oracle)
    for step in range(4):
        sm.step(1)
        kseq.cluster_step(be, sc, s, ())
        st = sm.state()
        for k in ("pos", "vel", "ep", "ev", "cpos"):
            scale = max(np.abs(s[k]).max(), 1e-300)
            assert np.abs(st[k] - s[k]).max() <= 1e-11 * scale, (step, k)
        cnt, ids, _ = sm.pairs(0)
        assert kseq.pairs_equal(cnt, ids, s["pp_count"], s["pp_id"], 12) == sc.np_


def test_caller_stream_survives_the_handle(simmod):
    """A stream given with xdem_sim_set_stream stays the caller's: destroying
    the handle must leave it usable for the next handle."""
    import torch
    from xdynamics_dll_gb300 import scenes
    sc = scenes.sphere_drop(n_per_layer_side=12, layers=2)
    stream = torch.cuda.Stream()
    ref = None
    for _ in range(2):
        s = simmod.Sim(sc, precision=T.XDEM_MIXED)
        s.L.xdem_sim_set_stream(s.h, stream.cuda_stream)
        s.set_graph(True)
        s.step(12)
        st = s.state()
        s.close()
        if ref is None:
            ref = st
        else:
            assert np.array_equal(ref["pos"], st["pos"])
    stream.synchronize()


def drum(n=1500, seed=31, cluster=False):
    """Spheres (or three-sphere clusters) in a cylinder of radius 20 mm,
    length 40 mm and 2 mm wall, open at the top, spinning slowly about its
    axis (y) and drifting, with random velocities: contacts with the inner
    wall, the base cap from inside and each other."""
    rng = np.random.default_rng(seed)
    L, R = 0.04, 0.02
    cyl = T.CylinderInfo()
    cyl.empty_part = 1
    cyl.thickness = 0.002
    cyl.len_rr = T.d3((L, R, R))
    cyl.pbase = T.d3((0.0, -0.5 * L, 0.0))
    cyl.ptop = T.d3((0.0, 0.5 * L, 0.0))
    body = T.body_record(mass=0.5, pos=(0.001, 0.002, -0.001), vel=(0.0, 0.0, 0.01), ed=(0.0, 0.0, 1.5, 0.0))
    if cluster:
        sc = scenes.cluster_bed(n // 3, neach=3, sub_r=1e-3, seed=seed, trough=(0.03, 0.03, 0.03),
                                spacing_factor=0.75, vel_scale=0.2)
        # the bed centred on the axis with its lowest members 0.2 mm into
        # the base, cluster centres spread by 1.2 about the axis (each
        # cluster moved rigidly) so that the outer members reach the wall
        p = sc.pos.reshape(-1, 3, 4)
        c = sc.cpos.reshape(-1, 4)
        low = np.array([p[..., 0].mean(), p[..., 1].min() - 0.8e-3, p[..., 2].mean()])
        shift = body[1:4] + np.array([0.0, -0.5 * L, 0.0]) - low
        p[..., :3] += shift
        c[:, :3] += shift
        move = np.zeros((c.shape[0], 3))
        move[:, [0, 2]] = 0.2 * (c[:, [0, 2]] - body[[1, 3]])
        c[:, :3] += move
        p[..., :3] += move[:, None, :]
        sc.pos, sc.cpos = p.ravel(), c.ravel()
    else:
        sc = scenes.random_packed(n, 0.8e-3, 1.2e-3, None, seed=seed, vel_scale=0.3)
        rho = R * np.sqrt(rng.uniform(0, 1, n)) * 0.97
        th = rng.uniform(0, 2 * np.pi, n)
        p = sc.pos.reshape(-1, 4).copy()
        p[:, 0] = body[1] + rho * np.cos(th)
        p[:, 2] = body[3] + rho * np.sin(th)
        p[:, 1] = body[2] + rng.uniform(-0.5 * L + 0.5e-3, 0.3 * L, n)
        sc.pos = p.ravel()
    sc.planes, sc.plane_cp, sc.plane_body = [], [], []
    sc.cylinders = [dict(cyl=cyl, body=body, cp=sc.pp_cp)]
    return sc


@pytest.mark.parametrize("cluster", [False, True])
def test_handle_with_cylinder_matches_oracle(simmod, oracle, cluster):
    """A handle with a cylinder (launcher kernels, FP64) against the oracle's
    step sequence with its cylinder contact (pinned to the reference's own
    cylinder kernels), six steps; pair lists exact, state to 1e-11."""
    sc = drum(cluster=cluster)
    sm = simmod.Sim(sc, precision=T.XDEM_FP64)
    s = kseq.state_arrays(sc)
    be = kseq.OracleBackend(oracle)
    touched = 0
    for step in range(6):
        sm.step(1)
        if cluster:
            kseq.cluster_step(be, sc, s, ())
        else:
            kseq.sphere_step(be, sc, s, (), compat=0)
        st = sm.state()
        for k in ("pos", "vel", "acc", "ep", "ev", "ea"):
            scale = max(np.abs(s[k]).max(), 1e-300)
            assert np.abs(st[k] - s[k]).max() <= 1e-11 * scale, (step, k)
        for kind, (ck, ik, cap) in ((0, ("pp_count", "pp_id", 12)), (3, ("cy_count", "cy_id", 3))):
            cnt, ids, _ = sm.pairs(kind)
            assert kseq.pairs_equal(cnt, ids, s[ck], s[ik], cap) == sc.np_, (step, ck)
        touched += int(s["cy_count"].sum())
    assert sm.status() == 0
    assert touched > 0
    w = sm.wrench(sm.bodies[0])
    assert np.abs(w).max() > 0


def test_mixed_handle_with_cylinder_matches_fp64(simmod):
    """The mixed step's cylinder contact (the FP64 regions of the launcher
    kernel, FP32 forces) against the FP64 handle on the spinning, drifting
    drum: after one step the particle-pair and cylinder pair lists are
    identical and the contact accelerations (force / mass) and Euler-parameter
    accelerations agree to 1e-4 of the largest, the cylinder's wrench to 1e-4;
    over 200 steps the kinetic energy to 1e-3 and the cylinder contacts stay
    equal."""
    sc = drum(n=1500)
    a = simmod.Sim(sc, precision=T.XDEM_FP64)
    b = simmod.Sim(sc, precision=T.XDEM_MIXED)
    a.step(1)
    b.step(1)
    sa, sb = a.state(), b.state()
    g = np.tile(np.array(sc.gravity), sc.np_)
    fa, fb = sa["acc"] - g, sb["acc"] - g
    assert np.abs(fa - fb).max() <= 1e-4 * np.abs(fa).max()
    assert np.abs(sa["ea"] - sb["ea"]).max() <= 1e-4 * np.abs(sa["ea"]).max()
    touched = 0
    for kind, cap in ((0, 12), (3, 3)):
        ca, ia, _ = a.pairs(kind)
        cb, ib, _ = b.pairs(kind)
        assert np.array_equal(ca, cb), kind
        ia, ib = ia.reshape(-1, cap), ib.reshape(-1, cap)
        for i in np.nonzero(ca)[0]:
            assert np.array_equal(ia[i, :ca[i]], ib[i, :ca[i]]), (kind, i)
        if kind == 3:
            touched = int(ca.sum())
    assert touched > 0
    wa, wb = a.wrench(a.bodies[0]), b.wrench(b.bodies[0])
    for part in (slice(0, 3), slice(3, 6)):
        assert np.abs(wa[part] - wb[part]).max() <= 1e-4 * np.abs(wa[part]).max(), (wa, wb)
    a.step(199)
    b.step(199)
    ka, _ = a.energy()
    kb, _ = b.energy()
    assert abs(ka - kb) <= 1e-3 * ka, (ka, kb)
    assert a.status() == 0 and b.status() == 0
    a.close()
    b.close()


def test_mixed_cluster_handle_with_cylinder_matches_fp64(simmod):
    """The mixed cluster step's cylinder contact (members with their
    cluster's mass, velocity and spin, moments about the cluster centre)
    against the FP64 cluster handle on the launcher kernels, on the spinning,
    drifting drum of three-sphere clusters: after one step the particle-pair
    and cylinder pair lists are identical, the contact accelerations and
    Euler-parameter accelerations agree to 1e-4 of the largest and the
    cylinder's wrench to 1e-4; over 100 steps the kinetic energy to 1e-3."""
    sc = drum(cluster=True)
    a = simmod.Sim(sc, precision=T.XDEM_FP64)
    b = simmod.Sim(sc, precision=T.XDEM_MIXED)
    a.step(1)
    b.step(1)
    assert a.status() == 0 and b.status() == 0
    sa, sb = a.state(), b.state()
    g = np.asarray(sc.gravity, dtype=np.float64)
    fa, fb = sa["acc"].reshape(-1, 3) - g, sb["acc"].reshape(-1, 3) - g
    assert np.abs(fa - fb).max() <= 1e-4 * np.abs(fa).max()
    assert np.abs(sa["ea"] - sb["ea"]).max() <= 1e-4 * np.abs(sa["ea"]).max()
    touched = 0
    for kind, cap in ((0, 12), (3, 3)):
        ca, ia, _ = a.pairs(kind)
        cb, ib, _ = b.pairs(kind)
        assert kseq.pairs_equal(cb, ib, ca, ia, cap) == sc.np_, kind
        if kind == 3:
            touched = int(ca.sum())
    assert touched > 0
    wa, wb = a.wrench(a.bodies[0]), b.wrench(b.bodies[0])
    for part in (slice(0, 3), slice(3, 6)):
        assert np.abs(wa[part] - wb[part]).max() <= 1e-4 * np.abs(wa[part]).max(), (wa, wb)
    a.step(99)
    b.step(99)
    ka, _ = a.energy()
    kb, _ = b.energy()
    assert abs(ka - kb) <= 1e-3 * ka, (ka, kb)
    assert a.status() == 0 and b.status() == 0
    a.close()
    b.close()


@pytest.mark.parametrize("nt", [64, 128, 256])
def test_mixed_plane_wrench_rows_with_padding_warps(simmod, nt):
    """1,100 spheres in an open box, numbered so that the first 64 rest on
    the wall x = x0 (plane 1): the body kernel's last block holds padding
    warps past the last sphere, which must leave the per-warp wrench rows of
    the next plane alone.  Every plane's wrench of the mixed step against the
    FP64 step on the same state, to 1e-4 of its size."""
    sc = scenes.random_packed(1100, 0.8e-3, 1.2e-3, None, seed=21)
    order = np.argsort(sc.pos.reshape(-1, 4)[:, 0], kind="stable")  # spheres nearest the wall x = x0 first
    for key, w in (("pos", 4), ("vel", 3), ("acc", 3), ("ep", 4), ("ev", 4), ("ea", 4), ("mass", 1),
                   ("inertia", 3)):
        setattr(sc, key, np.asarray(getattr(sc, key)).reshape(-1, w)[order].ravel())
    a = simmod.Sim(sc, precision=T.XDEM_FP64)
    b = simmod.Sim(sc, precision=T.XDEM_MIXED)
    b.set_tune(nt_pairs=nt, stage=16, nt_bodies=nt, occ_pairs=768, occ_bodies=768, skin_div=0)
    a.step(1)
    b.step(1)
    touched = 0
    for body in a.bodies:
        wa, wb = a.wrench(body), b.wrench(body)
        for part in (slice(0, 3), slice(3, 6)):
            s_ = np.abs(wa[part]).max()
            if s_ > 0:
                touched += 1
                assert np.abs(wa[part] - wb[part]).max() <= 1e-4 * s_, (body, wa, wb)
    assert touched >= 4
    a.close()
    b.close()


def test_cylinder_pairs_survive_a_part_file(simmod, tmp_path):
    """save_part writes the cylinder block between the plane and triangle
    blocks (xResultManager.cpp:897-902); a handle loaded from it continues
    bit for bit."""
    from xdynamics_dll_gb300 import partfile
    sc = drum(n=800, seed=5)
    a = simmod.Sim(sc, precision=T.XDEM_FP64)
    a.step(5)
    path = tmp_path / "cyl.bin"
    a.save_part(path, 5e-5)
    d = partfile.read(path, kinds=("pp", "cy"))
    cnt, ids, tsd = a.pairs(3)
    assert np.array_equal(d["cy_count"], cnt) and np.array_equal(d["cy_id"], ids) and np.array_equal(d["cy_tsd"], tsd)
    assert cnt.sum() > 0
    b = simmod.Sim(sc, precision=T.XDEM_FP64)
    b.load_part(path)
    a.step(4)
    b.step(4)
    sa, sb = a.state(), b.state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
    a.close()
    b.close()


@pytest.mark.parametrize("launcher_path", [0, 1])
def test_rolling_inertia_per_sphere_matches_oracle(simmod, oracle, launcher_path):
    """xdem_sim_set_rolling_inertia(1): rolling resistance with each sphere's
    own inertia (the reference reads the flat entry i of the double3 array,
    impl:2434) against the oracle with the same switch; and the switch does
    change the motion."""
    sc = scene_with_mesh(seed=23, rfric=0.05)
    sm = simmod.Sim(sc, precision=T.XDEM_FP64, launcher_path=launcher_path)
    sm.set_rolling_inertia(1)
    ref = simmod.Sim(sc, precision=T.XDEM_FP64, launcher_path=launcher_path)
    meshes = oracle_meshes_from_sim(sm, sc)
    s = kseq.state_arrays(sc)
    s["rolling_per_sphere"] = 1
    be = kseq.OracleBackend(oracle)
    for step in range(5):
        sm.step(1)
        ref.step(1)
        kseq.sphere_step(be, sc, s, meshes, compat=0)
        compare(sm, s, sc, 1e-11, step)
    assert sm.status() == 0
    assert not np.array_equal(sm.state()["ev"], ref.state()["ev"])
    sm.close()
    ref.close()


@pytest.mark.parametrize("precision", [T.XDEM_FP64, T.XDEM_MIXED])
def test_batched_body_exchange_matches_per_body_calls(simmod, precision):
    """xdem_sim_set_bodies / xdem_sim_body_wrenches against one
    xdem_sim_set_body / xdem_sim_body_wrench call per body: five planes (their
    records given a sliding velocity, their frames re-sent) and a mesh pushed
    through the bed, re-posed every step; states and wrenches bit for bit."""
    sc = scene_with_mesh(seed=12)
    nb = len(sc.planes) + 1
    out = []
    for batched in (False, True):
        sm = simmod.Sim(sc, precision=precision)
        assert len(sm.bodies) == nb
        recs = np.array([np.asarray(r, dtype=np.float64) for r in sc.plane_body] +
                        [np.asarray(sc.meshes[0]["body"], dtype=np.float64)])
        walls = []
        for step in range(12):
            recs[:len(sc.planes), 4] = 0.01 * (step + 1)  # the planes slide along x
            recs[-1, 2] += 0.02 * sc.dt                   # the mesh moves along y
            if batched:
                sm.set_bodies(sm.bodies, recs, list(sc.planes) + [T.PlaneInfo()])
            else:
                for b in range(nb):
                    sm.set_body(sm.bodies[b], recs[b], sc.planes[b] if b < len(sc.planes) else None)
            sm.step(1)
            if batched:
                w = sm.wrenches(sm.bodies)
            else:
                w = np.array([sm.wrench(sm.bodies[b]) for b in range(nb)])
            walls.append(w)
        assert sm.status() == 0
        out.append((sm.state(), np.array(walls), [sm.pairs(k) for k in (0, 1, 2)]))
        sm.close()
    (sa, wa, pa), (sb, wb, pb) = out
    for k in ("pos", "vel", "acc", "ep", "ev", "ea"):
        assert np.array_equal(sa[k], sb[k]), k
    assert np.array_equal(wa, wb)
    assert np.abs(wa).max() > 0
    for x, y in zip(pa, pb):
        for u, v in zip(x, y):
            assert np.array_equal(u, v)


def test_batched_body_exchange_checks_its_arguments(simmod):
    sc = scene_with_mesh(n=500, seed=3)
    sm = simmod.Sim(sc, precision=T.XDEM_MIXED)
    with pytest.raises(Exception):
        sm.set_bodies([len(sm.bodies)], np.zeros((1, 15)))
    sm.step(1)
    assert sm.wrenches([]).shape == (0, 6)
    w = sm.wrenches([sm.bodies[-1], sm.bodies[0]])
    assert np.array_equal(w[0], sm.wrench(sm.bodies[-1]))
    assert np.array_equal(w[1], sm.wrench(sm.bodies[0]))
    sm.close()


@pytest.mark.parametrize("n_side", [1, 2])
def test_smallest_scenes_match_oracle(simmod, oracle, n_side):
    """One sphere, and a 2 x 2 layer, falling onto the floor of the drop's
    box: the handle (FP64) against the oracle over the fall and the first
    impacts, and the mixed form's kinetic energy against FP64."""
    sc = scenes.sphere_drop(n_per_layer_side=n_side, layers=1, dt=1e-5, box=0.02, wall_height=0.01)
    assert sc.np_ == n_side * n_side
    sm = simmod.Sim(sc, precision=T.XDEM_FP64)
    mx = simmod.Sim(sc, precision=T.XDEM_MIXED)
    s = kseq.state_arrays(sc)
    be = kseq.OracleBackend(oracle)
    hit = 0
    ke = []
    # the spheres start 2.2 mm above the floor: about 2,100 steps of fall
    for step in range(60):
        sm.step(50)
        mx.step(50)
        for _ in range(50):
            kseq.sphere_step(be, sc, s, [], compat=0)
        compare(sm, s, sc, 1e-9, step)
        hit += int(s["pl_count"].sum())
        ke.append((sm.energy()[0], mx.energy()[0]))
    assert hit > 0  # the spheres reached the floor
    ke = np.array(ke)
    # judged on the trace's scale: at a bounce's turning point the energy
    # itself is near zero
    assert np.abs(ke[:, 0] - ke[:, 1]).max() <= 1e-3 * ke[:, 0].max(), ke
    assert sm.status() == 0 and mx.status() == 0
