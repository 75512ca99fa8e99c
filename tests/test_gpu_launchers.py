"""GPU launchers (reference-named C-ABI) against the reference's own
kernels (golden fixtures) and the CPU oracle.

Bar: cell ids, sort order, cell ranges and pair lists bit-exact; floating
point within 1e-12 relative of the fixture scale (the FP64 launchers round
like the reference except pow(x, 1.5) -> x*sqrt(x) and the closed-form
Euler-parameter solve)."""
import numpy as np
import pytest

import kseq
from xdynamics_dll_gb300 import scenes, types as T

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from xdynamics_dll_gb300 import build, launchers
    build.build()
    return launchers.Launchers()


@pytest.mark.parametrize("kind", ["sphere", "cluster"])
def test_step_matches_reference_fixture(gpu, kind):
    sc, s, meshes, exp = kseq.load_ref_fixture(kind)
    gpu.forget()
    if kind == "sphere":
        g, st, _ = kseq.sphere_step(gpu, sc, s, meshes, compat=1)
    else:
        g, st, _ = kseq.cluster_step(gpu, sc, s, meshes)
    gpu.download()
    assert st == 0
    kseq.check_outputs(s, g, exp, kind=kind, ftol=1e-12)


def test_body_wrench_matches_partials(gpu, oracle):
    sc, s, meshes, exp = kseq.load_ref_fixture("sphere")
    # run up to the first plane on the GPU, then compare the summed wrench
    prm = sc.params()
    gpu.forget()
    gpu.set_params(prm)
    gpu.vv_pos(s)
    ntot = s["np"] + meshes[0]["ntri"]
    g = kseq.grid_arrays(prm, ntot)
    gpu.hash(g, s["pos"], 0, s["np"])
    gpu.hash(g, meshes[0]["sphere"], s["np"], meshes[0]["ntri"])
    gpu.reorder(g, ntot)
    gpu.p2p(s, g, sc.pp_cp)
    gpu.plane(s, sc.planes[0], np.asarray(sc.plane_body[0]), sc.plane_cp[0])
    w = gpu.last_wrench()
    ref = exp["partials"][0].sum(axis=1)
    assert np.allclose(w, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    # `reduction` (def:285-317) on one partial array
    gpu.download()
    assert np.isclose(gpu.reduction(s["bf"][1]), s["bf"][1].sum(), rtol=1e-12, atol=1e-15)


def _random_sphere_scene(seed, n=2500, rfric=0.0):
    sc = scenes.random_packed(n, 0.8e-3, 1.2e-3, None, seed=seed, rfric=rfric)
    return sc


@pytest.mark.parametrize("seed,compat", [(3, 0), (4, 1)])
def test_launchers_vs_oracle_random(gpu, oracle, seed, compat):
    sc = _random_sphere_scene(seed, rfric=0.02 * (seed % 2))
    s_gpu = kseq.state_arrays(sc)
    s_cpu = kseq.state_arrays(sc)
    be_cpu = kseq.OracleBackend(oracle)
    for step in range(3):
        gpu.forget()
        g1, st1, _ = kseq.sphere_step(gpu, sc, s_gpu, (), compat=compat)
        gpu.download()
        g2, st2, _ = kseq.sphere_step(be_cpu, sc, s_cpu, (), compat=compat)
        assert st1 == st2 == 0
        for k in ("hash", "index", "sorted_index", "cstart", "cend"):
            assert np.array_equal(g1[k], g2[k]), k
        assert kseq.pairs_equal(s_gpu["pp_count"], s_gpu["pp_id"], s_cpu["pp_count"], s_cpu["pp_id"], 12) == sc.np_
        assert kseq.pairs_equal(s_gpu["pl_count"], s_gpu["pl_id"], s_cpu["pl_count"], s_cpu["pl_id"], 3) == sc.np_
        for k in ("pos", "vel", "acc", "ep", "ev", "ea", "pp_tsd", "pl_tsd"):
            a, b = s_gpu[k], s_cpu[k]
            scale = max(np.abs(b).max(), 1e-300)
            assert np.abs(a - b).max() <= 1e-11 * scale, (step, k, np.abs(a - b).max(), scale)
    assert s_cpu["pp_count"].sum() > sc.np_ // 4  # the scene really is in contact
    assert s_cpu["pl_count"].sum() > 0


def test_overflow_sets_status_and_keeps_slots(gpu, oracle):
    # 40 equal spheres on top of each other: every sphere touches 39 others
    n = 40
    rng = np.random.default_rng(9)
    pos = np.zeros((n, 4))
    pos[:, :3] = rng.normal(0, 1e-5, size=(n, 3))
    pos[:, 3] = 1e-3
    m, J = scenes.sphere_mass_inertia(np.full(n, 1e-3), 2500.0)
    vel, acc, ep, ev, ea = scenes._init_state(n)
    sc = scenes.Scene(np_=n, ns=n, pos=pos.ravel(), vel=vel, acc=acc, ep=ep, ev=ev, ea=ea, mass=m,
                      inertia=J.ravel(), dt=1e-6, cell_size=2e-3, pp_cp=scenes.default_material())
    s_gpu, s_cpu = kseq.state_arrays(sc), kseq.state_arrays(sc)
    gpu.forget()
    _, st1, _ = kseq.sphere_step(gpu, sc, s_gpu, (), compat=0)
    gpu.download()
    _, st2, _ = kseq.sphere_step(kseq.OracleBackend(oracle), sc, s_cpu, (), compat=0)
    assert st1 & T.XDEM_ERR_P2P_OVERFLOW and st2 & T.XDEM_ERR_P2P_OVERFLOW
    assert np.all(s_gpu["pp_count"] == T.MAX_P2P_COUNT)
    assert np.array_equal(s_gpu["pp_id"], s_cpu["pp_id"])
    assert np.allclose(s_gpu["vel"], s_cpu["vel"], rtol=1e-12, atol=1e-15)
