"""The CPU oracle against the golden fixtures (no GPU).

part0104_kat.npz pins hash, stable sort, cell start/end, the cluster
contact search and the cluster plane slot rule against pair lists the
reference's GPU path wrote.  ref_sphere.npz / ref_cluster.npz pin every
kernel of the step against the reference's own kernels compiled for the
host (tests/golden/make_golden.py)."""
import numpy as np
import pytest

import kseq
from xdynamics_dll_gb300 import types as T


def test_part0104_pair_lists(oracle):
    d = np.load(kseq.GOLDEN + "/part0104_kat.npz")
    n, ns = int(d["np_"]), int(d["ns"])
    prm = T.make_params(np_=n, dt=1e-5, cell_size=float(d["cell_size"]), ncluster=ns, nco=1, nplane=6)
    cp = T.make_contact_property(E_i=1e7, E_j=1e7, nu_i=0.3, nu_j=0.3, rest=0.5, fric=0.3)
    xci = d["xci"].copy()
    pos, cpos = d["pos"].copy(), d["cpos"].copy()
    vel, ep, ev, mass = d["vel"].copy(), d["ep"].copy(), d["ev"].copy(), d["mass"].copy()
    g = kseq.grid_arrays(prm, n)
    assert oracle.hash(prm, g["hash"], g["index"], pos, 0, n) == 0
    oracle.reorder(g["hash"], g["index"], g["cstart"], g["cend"], g["sorted_index"], n, prm.ncell)
    assert np.all(np.diff(g["hash"].astype(np.int64)) >= 0)
    force, mom, tmax, rres = (np.zeros(n * 3), np.zeros(n * 3), np.zeros(n * 3), np.zeros(n))
    pc, pid, tsd = np.zeros(n, np.uint32), np.zeros(n * 12, np.uint32), np.zeros(n * 24)
    st = oracle.clusters_p2p(prm, pos, cpos, ep, vel, ev, force, mom, mass, tmax, rres, pc, pid, tsd,
                             g["sorted_index"], g["cstart"], g["cend"], cp, xci, n)
    assert st == 0
    assert kseq.pairs_equal(pc, pid, d["pp_count"], d["pp_id"], 12) == n
    lc, lid, ltsd = np.zeros(n, np.uint32), np.zeros(n * 3, np.uint32), np.zeros(n * 6)
    bf = [np.zeros(n) for _ in range(6)]
    for pl in T.cube_planes(d["cube_min"], d["cube_max"]):
        oracle.cluster_plane(prm, pl, T.body_record(), bf, pos, cpos, ep, vel, ev, force, mom, cp, mass, tmax,
                             rres, lc, lid, ltsd, xci, n)
    assert kseq.pairs_equal(lc, lid, d["pl_count"], d["pl_id"], 3) == n
    assert int(pc.sum()) == int(d["pp_count"].sum()) == 11304


@pytest.mark.parametrize("kind", ["sphere", "cluster"])
def test_step_matches_reference_kernels(oracle, kind):
    sc, s, meshes, exp = kseq.load_ref_fixture(kind)
    be = kseq.OracleBackend(oracle)
    if kind == "sphere":
        g, st, partials = kseq.sphere_step(be, sc, s, meshes, compat=1)
    else:
        g, st, partials = kseq.cluster_step(be, sc, s, meshes)
    assert st == 0
    # the oracle solves the Euler-parameter equations with its own adjugate;
    # everything else follows the reference's operation order
    kseq.check_outputs(s, g, exp, kind=kind, ftol=1e-12)
    assert np.allclose(np.array([np.stack(p) for p in partials]), exp["partials"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("case", range(8))
def test_cylinder_matches_reference_kernels(oracle, case):
    """The oracle's cylinder contact (xo_cylinder) against the reference's
    own cylinder kernels (ref_cylinder.npz): every output bit for bit."""
    inp, cp, model, exp = kseq.load_cylinder_fixture()[case]

    def run(prm, cyl, body, cp, bf, s, p):
        return oracle.cylinder(prm, cyl, body, cp, bf, s["pos"], s["cpos"], s["ep"], s["vel"], s["ev"], s["force"],
                               s["moment"], s["mass"], s["tmax"], s["rres"], p["pair_count"], p["pair_id"], p["tsd"],
                               s["xci"], len(s["pos"]) // 4)

    out, st = kseq.run_cylinder(run, inp, cp, model)
    assert st == 0
    assert int(out["pair_count"].sum()) > 0
    for k, v in exp.items():
        assert np.array_equal(out[k], v), k
