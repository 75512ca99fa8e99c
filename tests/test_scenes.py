"""Host-side scene setup against the reference's formulas (no GPU)."""
import numpy as np

from xdynamics_dll_gb300 import scenes


def reference_cluster_mass_inertia(rloc, r, rho):
    """xParticleManager::SetClusterMassAndInertia
    (source/xdynamics_manager/xParticleManager.cpp:1071-1084), written out
    loop by loop: m = rho 4/3 pi r^3; mass = m * each; J3 sums, per member,
    m (dy^2 + dz^2, dx^2 + dz^2, dx^2 + dy^2) of its offset."""
    m = rho * (4.0 / 3.0) * np.pi * r ** 3.0
    J3 = [0.0, 0.0, 0.0]
    for dx, dy, dz in rloc:
        J3[0] += m * (dy * dy + dz * dz)
        J3[1] += m * (dx * dx + dz * dz)
        J3[2] += m * (dx * dx + dy * dy)
    return m * len(rloc), np.array(J3)


def test_clump_mass_and_inertia_follow_the_reference():
    # a tetrahedral four-sphere clump (the reference's part0104 clusters are
    # four-sphere clumps): every axis has a parallel-axis term
    r = 1.5e-3
    rloc = np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], float) * 0.8 * r
    m, J, own = scenes.cluster_mass_inertia(rloc, r, 2500.0)
    mr, Jr = reference_cluster_mass_inertia(rloc, r, 2500.0)
    assert m == mr and np.array_equal(J, Jr) and not own.any()


def test_row_clump_gets_only_the_missing_axis():
    # three spheres in a row along x: the reference's sum is zero about x;
    # only that axis takes the members' own 2/5 m r^2
    r = 2e-3
    rloc = np.array([[-1.9, 0, 0], [0, 0, 0], [1.9, 0, 0]]) * r
    m, J, own = scenes.cluster_mass_inertia(rloc, r, 2500.0)
    mr, Jr = reference_cluster_mass_inertia(rloc, r, 2500.0)
    assert m == mr and Jr[0] == 0.0
    assert own.tolist() == [True, False, False]
    assert J[1] == Jr[1] and J[2] == Jr[2]
    assert np.isclose(J[0], 3 * 0.4 * (2500.0 * 4.0 / 3.0 * np.pi * r ** 3) * r * r, rtol=1e-15)


def test_cluster_scenes_use_the_reference_setup():
    sc = scenes.cluster_bed(50, neach=3)
    rloc = sc.rloc.reshape(-1, 3)
    m, J, _ = scenes.cluster_mass_inertia(rloc, 2e-3, 2500.0)
    assert np.all(sc.mass == m) and np.array_equal(sc.inertia.reshape(-1, 3)[0], J)
