"""The adjoint's hand-written VJPs (xdynamics_dll_gb300/csrc/xdem_adjoint.cuh)
against central differences of their forward functions, on the host.

The header is plain C++ outside nvcc, so g++ builds tests/adjoint_vjp_check.cpp
into a small program; each line it prints is one VJP and the largest
relative error over 12 random directions.  Covered: angular velocity, body
rotation, the Euler-parameter acceleration (anisotropic and isotropic
inertia) and the torque recovered from it, normalisation, a sphere's
particle-particle contacts (Hertz-Mindlin and DHS, stick and slip, a contact
that keeps the previous tangential force) and plane contacts in the face,
edge and corner regions.  The same forward pieces evaluated on dual numbers
(forward mode) are checked against the VJPs and the differences too.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def results(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path_factory.mktemp("adj") / "adjoint_vjp_check")
    subprocess.run([cxx, "-O1", "-std=c++17", "-o", exe, os.path.join(HERE, "adjoint_vjp_check.cpp")], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    errs, notes = {}, {}
    for line in out.splitlines():
        if line.startswith("#"):
            f = line[1:].split()
            notes[f[0]] = f[1:]
        else:
            name, val = line.split()
            errs[name] = float(val)
    return errs, notes


def test_all_vjps_match_central_differences(results):
    errs, _ = results
    expected = {"ang_vel", "to_local", "uceom", "uceom_isotropic", "normalize", "pp_hm", "pp_dhs", "pp_hm_kept_ft",
                "plane_face_hm", "plane_face_dhs", "plane_edge_hm", "plane_corner_hm"}
    assert expected <= set(errs)
    bad = {k: v for k, v in errs.items() if k in expected and not v < 1e-6}
    assert not bad, bad


def test_dual_number_tangents_match_vjps_and_differences(results):
    """The forward pieces on dual numbers (the forward mode the tangent
    kernels run): ly . (J d) against (VJP ly) . d and central differences."""
    errs, _ = results
    expected = {k + "_jvp" for k in ("ang_vel", "to_local", "uceom", "uceom_isotropic", "normalize", "pp_hm", "pp_dhs",
                                     "pp_hm_kept_ft", "plane_face_hm", "plane_face_dhs", "plane_edge_hm",
                                     "plane_corner_hm")}
    assert expected <= set(errs)
    bad = {k: v for k, v in errs.items() if k in expected and not v < 1e-6}
    assert not bad, bad


def test_uceom_torque_inverts_the_solve(results):
    errs, _ = results
    assert errs["uceom_torque"] < 1e-12 and errs["uceom_torque_isotropic"] < 1e-12


def test_cases_cover_the_regimes(results):
    _, notes = results

    def counts(name):
        f = notes[name]
        return {f[i]: int(f[i + 1]) for i in range(0, len(f), 2)}

    hm = counts("pp_hm")
    assert hm["stick"] >= 1 and hm["slip"] >= 1
    assert counts("pp_hm_kept_ft")["kept"] == 1
    assert notes["plane_face_hm"][1] == "3"
    assert notes["plane_edge_hm"][1] == "2"
    assert notes["plane_corner_hm"][1] == "1"
