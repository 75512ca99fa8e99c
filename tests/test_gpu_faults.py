"""Failure detection by host-side injection: corrupt part files, corrupt
pair lists, non-finite state and forced pair-list overflow.

Every fault is made on the host (a damaged file, a bad array handed to the
C-ABI, a scene whose geometry exceeds a capacity).  The library must refuse
bad input before it reaches the device, leaving the handle as it was, or
flag a device-side condition in its status word and keep every write inside
the lists' slots.  Nothing here faults, traps or hangs a GPU: the only values
a kernel sees are finite in-range states, plus one NaN position handed to
the hash launcher, whose conversion saturates into the grid and raises
XDEM_ERR_NONFINITE."""
import ctypes as C
import os

import numpy as np
import pytest

from xdynamics_dll_gb300 import partfile, scenes, types as T

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from xdynamics_dll_gb300 import build, sim, _lib
    build.build()
    return torch, sim, _lib.lib()


def small_drop():
    """300 overlapping spheres in a box of five planes: particle-pair and
    plane contacts from the first step."""
    return scenes.random_packed(300, 0.8e-3, 1.2e-3, None, seed=5)


def snapshot(sm):
    st = sm.state()
    return st, [sm.pairs(k) for k in range(2)]


def same(a, b):
    """Bit-for-bit equality of two snapshots (slots past a sphere's count
    hold whatever the allocation held, possibly NaN patterns, so values are
    compared as bytes)."""
    (sa, pa), (sb, pb) = a, b
    eq = lambda x, y: x.shape == y.shape and x.tobytes() == y.tobytes()
    return all(eq(sa[k], sb[k]) for k in sa) and all(eq(x, y) for u, v in zip(pa, pb) for x, y in zip(u, v))


@pytest.fixture(scope="module")
def saved(env, tmp_path_factory):
    """A handle stepped into contact, its part file, and the file's blocks."""
    torch, sim, L = env
    sc = small_drop()
    sm = sim.Sim(sc, precision=T.XDEM_FP64)
    sm.step(6)
    assert sm.status() == 0
    path = str(tmp_path_factory.mktemp("part") / "good.part")
    sm.save_part(path, 6 * sc.dt)
    d = partfile.read(path, ("pp", "pl"))
    assert d["pp_count"].sum() > 0 and d["pl_count"].sum() > 0
    sm.close()
    return sc, path, d


def load_rc(sim, sc, L, path):
    """Loads `path` into a handle stepped twice; returns the return code and
    whether the handle's state and lists stayed as they were."""
    sm = sim.Sim(sc, precision=T.XDEM_FP64)
    sm.step(2)
    before = snapshot(sm)
    t = C.c_double()
    rc = L.xdem_sim_load_part(sm.h, path.encode(), C.byref(t))
    after = snapshot(sm)
    sm.close()
    return rc, same(before, after)


def test_good_part_file_loads(env, saved):
    torch, sim, L = env
    sc, path, _ = saved
    rc, unchanged = load_rc(sim, sc, L, path)
    assert rc == 0 and not unchanged


def test_truncated_part_file_is_refused(env, saved, tmp_path):
    torch, sim, L = env
    sc, path, _ = saved
    b = open(path, "rb").read()
    for cut in (7, 100, len(b) // 2, len(b) - 1):
        bad = str(tmp_path / f"cut{cut}.part")
        open(bad, "wb").write(b[:cut])
        rc, unchanged = load_rc(sim, sc, L, bad)
        assert rc == T.XDEM_ERR_ARG and unchanged, cut
    # one byte too many is refused too
    bad = str(tmp_path / "long.part")
    open(bad, "wb").write(b + b"\0")
    rc, unchanged = load_rc(sim, sc, L, bad)
    assert rc == T.XDEM_ERR_ARG and unchanged


@pytest.mark.parametrize("fault", ["pp_count", "pp_id", "pl_count", "pl_id"])
def test_corrupt_pair_block_is_refused(env, saved, tmp_path, fault):
    torch, sim, L = env
    sc, path, d = saved
    e = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in d.items()}
    n = sc.np_
    if fault == "pp_count":
        e["pp_count"][n // 2] = T.MAX_P2P_COUNT + 1          # a bit-flipped count beyond the slots
    elif fault == "pp_id":
        i = int(np.flatnonzero(e["pp_count"])[0])
        e["pp_id"][i * T.MAX_P2P_COUNT] = n                   # partner id past the last particle
    elif fault == "pl_count":
        e["pl_count"][0] = 1 << 20
    else:
        i = int(np.flatnonzero(e["pl_count"])[0])
        e["pl_id"][i * T.MAX_P2PL_COUNT] = len(sc.planes)     # a plane the model does not have
    bad = str(tmp_path / f"{fault}.part")
    partfile.write(bad, e, ("pp", "pl"))
    rc, unchanged = load_rc(sim, sc, L, bad)
    assert rc == T.XDEM_ERR_ARG and unchanged


def test_set_pairs_checks_counts_and_ids(env):
    torch, sim, L = env
    sc = small_drop()
    sm = sim.Sim(sc, precision=T.XDEM_MIXED)
    sm.step(3)
    before = snapshot(sm)
    n = sc.np_
    cnt, ids, tsd = sm.pairs(0)
    for mutate in ("count", "id", "stale_id_beyond_count"):
        c2, i2 = cnt.copy(), ids.copy()
        if mutate == "count":
            c2[1] = T.MAX_P2P_COUNT + 1
            expect = T.XDEM_ERR_ARG
        elif mutate == "id":
            c2[1] = max(c2[1], 1)
            i2[1 * T.MAX_P2P_COUNT] = n + 7
            expect = T.XDEM_ERR_ARG
        else:
            # ids in slots past a sphere's count are never read: accepted
            c2[1] = 0
            i2[1 * T.MAX_P2P_COUNT:2 * T.MAX_P2P_COUNT] = 0xFFFFFFFF
            expect = 0
        p = lambda a: C.c_void_p(np.ascontiguousarray(a).ctypes.data)
        rc = L.xdem_sim_set_pairs(sm.h, 0, p(c2), p(i2), p(tsd))
        assert rc == expect, mutate
        if expect:
            assert same(before, snapshot(sm)), mutate
    sm.close()


def test_nonfinite_state_is_refused_before_upload(env):
    torch, sim, L = env
    sc = small_drop()
    for prec in (T.XDEM_FP64, T.XDEM_MIXED):
        sm = sim.Sim(sc, precision=prec)
        sm.step(2)
        before = snapshot(sm)
        for key, val in (("pos", np.nan), ("vel", np.inf), ("mass", -np.inf)):
            arrs = {k: getattr(sc, k).copy() for k in ("pos", "vel", "acc", "ep", "ev", "ea", "mass", "inertia")}
            arrs[key][5] = val
            a = [np.ascontiguousarray(arrs[k], np.float64) for k in ("pos", "vel", "acc", "ep", "ev", "ea", "mass",
                                                                     "inertia")]
            rc = L.xdem_sim_set_state(sm.h, *[C.c_void_p(x.ctypes.data) for x in a])
            assert rc == T.XDEM_ERR_NONFINITE | T.XDEM_ERR_ARG, (prec, key)
            assert same(before, snapshot(sm)), (prec, key)
        sm.step(1)  # the handle stays usable
        assert sm.status() == 0
        sm.close()


def test_nan_position_in_hash_launcher_flags_and_stays_in_grid(env):
    torch, sim, L = env
    n = 1000
    rng = np.random.default_rng(3)
    pos = np.zeros((n, 4))
    pos[:, :3] = rng.uniform(-0.05, 0.05, size=(n, 3))
    pos[:, 3] = 1e-3
    pos[17, 0] = np.nan
    pos[18, 1] = np.inf
    prm = T.make_params(np_=n, dt=1e-5, cell_size=2e-3, grid=(128, 128, 128), origin=(-1.0, -1.0, -1.0),
                        gravity=(0.0, -9.80665, 0.0), contact_model=1)
    assert L.setDEMSymbolicParameter(C.byref(prm)) == 0
    L.xdem_take_device_status()
    dpos = torch.from_numpy(pos.ravel()).cuda()
    dh = torch.zeros(n, dtype=torch.int32, device="cuda")
    di = torch.zeros(n, dtype=torch.int32, device="cuda")
    rc = L.cu_calculateHashAndIndex(C.c_void_p(dh.data_ptr()), C.c_void_p(di.data_ptr()),
                                    C.c_void_p(dpos.data_ptr()), 0, n)
    torch.cuda.synchronize()
    assert rc == 0
    st = L.xdem_take_device_status()
    assert st & T.XDEM_ERR_NONFINITE
    h = dh.cpu().numpy().view(np.uint32)
    assert h.max() < 128 ** 3
    assert np.array_equal(di.cpu().numpy(), np.arange(n))
    assert L.xdem_take_device_status() == 0  # taking the status cleared it


@pytest.mark.parametrize("prec", [T.XDEM_FP64, T.XDEM_MIXED])
def test_forced_pair_overflow_is_flagged_and_bounded(env, prec):
    """40 spheres packed into one point: each touches 39 others, more than a
    particle-pair list holds.  The step flags XDEM_ERR_P2P_OVERFLOW, keeps
    MAX_P2P_COUNT entries per sphere, and the handle runs on normally once a
    valid state is loaded."""
    torch, sim, L = env
    n = 40
    rng = np.random.default_rng(9)
    pos = np.zeros((n, 4))
    pos[:, :3] = rng.normal(0, 1e-5, size=(n, 3))
    pos[:, 3] = 1e-3
    m, J = scenes.sphere_mass_inertia(np.full(n, 1e-3), 2500.0)
    vel, acc, ep, ev, ea = scenes._init_state(n)
    sc = scenes.Scene(np_=n, ns=n, pos=pos.ravel(), vel=vel, acc=acc, ep=ep, ev=ev, ea=ea, mass=m,
                      inertia=J.ravel(), dt=1e-6, cell_size=2e-3, pp_cp=scenes.default_material())
    sm = sim.Sim(sc, precision=prec)
    sm.step(1)
    assert sm.status() & T.XDEM_ERR_P2P_OVERFLOW
    cnt, ids, _ = sm.pairs(0)
    assert np.all(cnt == T.MAX_P2P_COUNT)
    # each stored partner is a real, distinct other sphere
    for i in range(n):
        row = ids[i * T.MAX_P2P_COUNT:(i + 1) * T.MAX_P2P_COUNT]
        assert np.all(row < n) and i not in row and len(set(row.tolist())) == T.MAX_P2P_COUNT
    assert np.all(np.isfinite(sm.state()["vel"]))
    # spread the spheres out: the next steps run clean
    p2 = pos.copy()
    p2[:, 0] = np.arange(n) * 3e-3
    p2[:, 1:3] = 0.0
    sm.set_state(p2.ravel(), None, acc, ep, None, None, m, J.ravel())
    sm.step(2)
    assert sm.status() == 0
    cnt, _, _ = sm.pairs(0)
    assert cnt.sum() == 0
    sm.close()
