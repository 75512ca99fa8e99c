"""Model workbooks (.xls): the BIFF8 cell reader and the model reader
against the reference's own workbooks (read where the reference tree sits
beside this repository, or at XDEM_REFERENCE_ROOT), and the scene built
from the committed cells of resource/cube_particle/cube_particle.xls
(tests/golden/make_xls_fixture.py), which the GPU test steps against the
oracle."""
import glob
import json
import os

import numpy as np
import pytest

from xdynamics_dll_gb300 import xls, xls_model as XM

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("XDEM_REFERENCE_ROOT") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
RES = os.path.join(REF, "resource")


def need(path):
    if not os.path.exists(path):
        pytest.skip("the reference's workbooks are not available (XDEM_REFERENCE_ROOT)")
    return path


def fixture_cells():
    d = json.load(open(os.path.join(HERE, "golden", "xls_cube_particle_cells.json")))
    return {(r, c): v for r, c, v in d["cells"]}


def test_wheel_testbed_workbook_reads_as_the_reference_reads_it():
    p = need(os.path.join(RES, "WheelTestBedWithCluster", "Wheeltestbedcluster_drive_JJS(14_0.2_3).xls"))
    m = XM.read_model(p)
    # section index of row 0 (one-based "row,col" cells)
    assert m["index"]["SHAPE"] == (2, 0) and m["index"]["PARTICLE"] == (7, 0) and m["index"]["CONTACT"] == (10, 0)
    cube = m["shapes"][0]
    # the box of the part0104 known-answer check
    assert cube["type"] == XM.CUBE and cube["p0"] == [-1.045, -0.1, -0.13] and cube["p1"] == [-0.345, 0.4, 0.13]
    assert m["shapes"][1]["type"] == XM.MESH and m["shapes"][1]["refinement"] == 0.00125
    p2p = m["contacts"][0]
    assert (p2p["model"], p2p["rest"], p2p["rto"], p2p["mu_s"], p2p["mu"], p2p["coh"], p2p["rf"]) == \
        (0, 0.2, 1.0, 0.0, 0.2, 0.0, 0.0)
    assert m["simulation"] == {"device": "GPU", "dt": 2e-06, "save_step": 1000.0, "end_time": 1.0}
    part = m["particles"][0]
    assert part["type"] == XM.CLUSTER and part["source"] == "cmf" and part["material"] == 7
    assert part["location"] == [-1.04, -0.09, -0.125]
    # the multibody rows come through as read: the drive joint's row
    assert m["joint"][0][:4] == ["rev", 2.0, "ground", "cube"]
    with pytest.raises(XM.XlsModelError, match="cmf"):
        XM.scene_from_model(m)


def test_old_layout_is_refused_as_the_reference_refuses_it():
    # its contact rows hold five numbers; ReadContactData reads six
    p = need(os.path.join(RES, "dem_dam_breaking.xls"))
    with pytest.raises(XM.XlsModelError, match="is not number type"):
        XM.read_model(p)


def test_reference_workbooks_read_or_fail_like_the_reference():
    need(RES)
    n_ok = n_all = 0
    for f in glob.glob(os.path.join(RES, "**", "*.xls"), recursive=True):
        cells = xls.read_cells(f)          # every workbook's cells read
        assert cells[(0, 0)] == "MODEL", f
        n_all += 1
        try:
            XM.model_from_cells(cells, f)
            n_ok += 1
        except XM.XlsModelError:
            pass                            # ReadStr / ReadNum throw there too
    assert n_all > 100 and n_ok >= 40, (n_all, n_ok)


def test_cylinder_and_mesh_rows_make_scene_bodies():
    p = need(os.path.join(RES, "cylinder_contact_test", "cylinder_contact_test.xls"))
    m = XM.read_model(p)
    sc = XM.scene_from_model(m)
    assert len(sc.cylinders) == 1
    cyl = sc.cylinders[0]["cyl"]
    s = [x for x in m["shapes"] if x["type"] == XM.CYLINDER][0]
    mid = 0.5 * (np.array(s["p0"]) + np.array(s["p1"]))
    assert np.allclose(sc.cylinders[0]["body"][1:4], mid)
    assert np.allclose([cyl.pbase.x, cyl.pbase.y, cyl.pbase.z], np.array(s["p0"]) - mid)
    assert (cyl.len_rr.x, cyl.len_rr.y, cyl.len_rr.z) == (s["length"], s["r_top"], s["r_bottom"])
    p = need(os.path.join(RES, "sphere_drop", "sphere_drop.xls"))
    sc = XM.scene_from_model(XM.read_model(p), base_dir=RES)
    assert len(sc.meshes) == 1 and sc.meshes[0]["vlist_local"].shape == (2400, 9)


def test_cube_fill_scene_from_the_committed_cells():
    m = XM.model_from_cells(fixture_cells(), "cube_particle.xls")
    sc = XM.scene_from_model(m, seed=3)
    part = m["particles"][0]
    # GetNumCubeParticles: (dimension / diameter - 1) per axis
    n_axis = int(0.01 / 0.002) - 1
    assert sc.np_ == n_axis ** 3 == 64
    p = sc.pos.reshape(-1, 4)
    assert np.all(p[:, 3] == part["max_radius"])
    lo = np.array(part["location"])
    assert np.all(p[:, :3] > lo) and np.all(p[:, :3] < lo + np.array(part["dimension"]))
    # sand particles against an acrylic cube: the reference's table
    assert (sc.pp_cp.Ei, sc.pp_cp.Ej, sc.pp_cp.pri) == (4.0e7, 4.0e7, 0.3)
    assert sc.plane_cp[0].Ej == 3.2e9 and sc.plane_cp[0].prj == 0.37
    c = m["contacts"][0]
    assert (sc.pp_cp.rest, sc.pp_cp.fric, sc.pp_cp.s_fric, sc.pp_cp.sratio) == (c["rest"], c["mu"], c["mu_s"],
                                                                                c["rto"])
    assert len(sc.planes) == 6 and sc.contact_model == 0 and sc.dt == 1e-6
    # the cube's six planes face inward (u1 x u2 toward the centre)
    centre = 0.5 * (np.array(m["shapes"][0]["p0"]) + np.array(m["shapes"][0]["p1"]))
    for pl in sc.planes:
        xw = np.array([pl.xw.x, pl.xw.y, pl.xw.z])
        uw = np.array([pl.uw.x, pl.uw.y, pl.uw.z])
        assert np.dot(centre - xw, uw) > 0


@pytest.mark.gpu
def test_workbook_scene_steps_as_the_oracle(oracle):
    """The scene of cube_particle.xls (64 sand spheres settling in an
    acrylic box, DHS) through the FP64 handle and the oracle, 300 steps of
    its 1e-6 s: pair lists exact and the state within 1e-11 of its scale."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import kseq
    from xdynamics_dll_gb300 import build, sim
    build.build()
    sc = XM.scene_from_model(XM.model_from_cells(fixture_cells(), "cube_particle.xls"), seed=3)
    # set the fill down on the floor (1 um overlap) so the steps have contacts
    p = sc.pos.reshape(-1, 4)
    p[:, 1] -= p[:, 1].min() - (p[:, 3].min() - 1e-6)
    sm = sim.Sim(sc, precision=0)
    s = kseq.state_arrays(sc)
    be = kseq.OracleBackend(oracle)
    touched = 0
    for k in range(300):
        sm.step(1)
        kseq.sphere_step(be, sc, s, (), compat=0)
        if k % 30 == 0:
            cnt, ids, _ = sm.pairs(1)
            assert kseq.pairs_equal(cnt, ids, s["pl_count"], s["pl_id"], 3) == sc.np_, k
            touched += int(s["pl_count"].sum())
    st = sm.state()
    for key in ("pos", "vel", "ep", "ev"):
        scale = max(np.abs(s[key]).max(), 1e-300)
        assert np.abs(st[key] - s[key]).max() <= 1e-11 * scale, key
    assert touched > 0 and sm.status() == 0
