"""Particle-cylinder contact launchers (cu_cylinder_contact_force,
cu_cluster_cylinder_contact; impl:1083-1601) against the CPU oracle, which
tests/test_oracle_golden.py pins bit for bit to the reference's own kernels
(tests/golden/ref_cylinder.npz).  FP64; the rim point goes through atan,
sin and cos, whose CUDA and host results may differ in the last place."""
import numpy as np
import pytest
import torch

import kseq
from xdynamics_dll_gb300 import scenes
from xdynamics_dll_gb300 import types as T

pytestmark = pytest.mark.gpu

CASES = [(1, 0.0, 0.0), (0, 0.0, 0.0), (1, 0.2, 0.0), (1, 0.0, 5e4)]


@pytest.fixture(scope="module")
def gl():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from xdynamics_dll_gb300 import build, launchers
    build.build()
    return launchers.Launchers()


def gpu_runner(gl):
    def run(prm, cyl, body, cp, bf, s, p):
        gl.forget()
        gl.set_params(prm)
        st = dict(s, np=len(s["pos"]) // 4, bf=bf, cy_count=p["pair_count"], cy_id=p["pair_id"],
                  cy_tsd=p["tsd"])
        status = gl.cylinder(st, cyl, body, cp)
        gl.download()
        return status
    return run


def oracle_runner(oracle):
    def run(prm, cyl, body, cp, bf, s, p):
        return oracle.cylinder(prm, cyl, body, cp, bf, s["pos"], s["cpos"], s["ep"], s["vel"], s["ev"],
                               s["force"], s["moment"], s["mass"], s["tmax"], s["rres"], p["pair_count"],
                               p["pair_id"], p["tsd"], s["xci"], len(s["pos"]) // 4)
    return run


def compare(a, b, n):
    assert kseq.pairs_equal(a["pair_count"], a["pair_id"], b["pair_count"], b["pair_id"], T.MAX_P2CY_COUNT) == n
    # torque-like arrays are judged on the scale of the contact moments: with
    # no rolling friction tmax holds only rounding residue (~1e-17)
    floor = {k: np.abs(b["moment"]).max() for k in ("tmax", "mx", "my", "mz")}
    for k in ("force", "moment", "tmax", "rres", "tsd", "fx", "fy", "fz", "mx", "my", "mz"):
        scale = max(np.abs(b[k]).max(), floor.get(k, 0.0), 1e-300)
        assert np.abs(a[k] - b[k]).max() <= 1e-12 * scale, (k, np.abs(a[k] - b[k]).max(), scale)


@pytest.mark.parametrize("cluster", [False, True])
@pytest.mark.parametrize("model,rf,coh", CASES)
def test_cylinder_launcher_matches_oracle(gl, oracle, cluster, model, rf, coh):
    inp = kseq.cylinder_inputs(3 + model, cluster=cluster)
    cp = scenes.default_material(rfric=rf)
    cp.coh = coh
    a, sa = kseq.run_cylinder(gpu_runner(gl), inp, cp, model)
    b, sb = kseq.run_cylinder(oracle_runner(oracle), inp, cp, model)
    assert sa == sb == 0
    assert (b["pair_id"].reshape(-1, 3)[b["pair_count"] > 0] >= 1000).any()  # inner caps reached
    compare(a, b, inp["n"])


def test_second_cylinder_appends_and_flags_overflow(gl, oracle):
    """A cylinder with id 1 appends after the count the first left (the
    plane slot rule); a sphere that collects more than MAX_P2CY_COUNT contacts
    keeps the first three and raises XDEM_ERR_P2CY_OVERFLOW (the reference
    writes on into the next particle's slots)."""
    inp = kseq.cylinder_inputs(11)
    cp = scenes.default_material()
    first_a, _ = kseq.run_cylinder(gpu_runner(gl), inp, cp)
    first_b, _ = kseq.run_cylinder(oracle_runner(oracle), inp, cp)
    compare(first_a, first_b, inp["n"])
    inp2 = dict(inp, pair_count=first_b["pair_count"], pair_id=first_b["pair_id"], tsd=first_b["tsd"])
    inp2["cyl"] = T.CylinderInfo.from_buffer_copy(inp["cyl"])
    inp2["cyl"].id = 1
    a, sa = kseq.run_cylinder(gpu_runner(gl), inp2, cp)
    b, sb = kseq.run_cylinder(oracle_runner(oracle), inp2, cp)
    assert sa == sb
    assert (b["pair_count"] > first_b["pair_count"]).any()
    assert sb & T.XDEM_ERR_P2CY_OVERFLOW
    compare(a, b, inp["n"])
