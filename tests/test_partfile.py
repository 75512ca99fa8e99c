"""Part files on the host (xdynamics_dll_gb300.partfile): the version-2 layout
of xResultManager::export_step_data_to_file round-trips, and, where the
reference's own snapshot is available (XDEM_REFERENCE_ROOT), reading it
gives the committed known-answer fixture.  Also the C-ABI's argument checks."""
import ctypes as C
import os

import numpy as np
import pytest

from xdynamics_dll_gb300 import partfile
from xdynamics_dll_gb300 import types as T

HERE = os.path.dirname(os.path.abspath(__file__))


def random_part(rng, npart, ns, kinds):
    d = {"time": 0.125, "np": npart, "ns": ns, "mass": rng.random(ns), "pos": rng.random(npart * 4),
         "vel": rng.random(ns * 3), "acc": rng.random(ns * 3), "ep": rng.random(ns * 4), "ev": rng.random(ns * 4),
         "ea": rng.random(ns * 4)}
    if npart != ns:
        d["cpos"] = rng.random(ns * 4)
    for k in kinds:
        cap = partfile.CAPS[k]
        d[k + "_count"] = rng.integers(0, cap + 1, npart).astype(np.uint32)
        d[k + "_id"] = rng.integers(0, npart, npart * cap).astype(np.uint32)
        d[k + "_tsd"] = rng.random(npart * cap * 2)
    return d


@pytest.mark.parametrize("npart,ns,kinds", [(50, 50, ("pp", "pl")), (60, 60, ("pp", "pl", "ms")),
                                             (90, 30, ("pp", "pl")), (40, 40, ("pp",))])
def test_round_trip(tmp_path, npart, ns, kinds):
    d = random_part(np.random.default_rng(npart), npart, ns, kinds)
    p = tmp_path / "part0001.bin"
    partfile.write(p, d, kinds)
    size = 8 + 8 + 8 * (ns + npart * 4 + ns * 3 * 2 + ns * 4 * 3 + (ns * 4 if npart != ns else 0))
    size += sum(npart * 4 + npart * 4 * partfile.CAPS[k] + npart * 16 * partfile.CAPS[k] for k in kinds)
    assert os.path.getsize(p) == size
    e = partfile.read(p, kinds)
    for k, v in d.items():
        assert np.array_equal(np.asarray(v), np.asarray(e[k])), k
    with pytest.raises(ValueError):
        partfile.read(p, kinds[:-1])  # a block the model does not have is left over


def test_reference_snapshot_reads_as_the_fixture():
    # the reference checkout sits beside this repository unless
    # XDEM_REFERENCE_ROOT says otherwise (it is absent where only the
    # committed fixtures travel)
    root = os.environ.get("XDEM_REFERENCE_ROOT") or os.path.join(os.path.dirname(os.path.dirname(HERE)),
                                                                 "reference")
    path = os.path.join(root, "resource", "input", "part0104.bin")
    if not os.path.exists(path):
        pytest.skip("the reference's snapshot is not available (XDEM_REFERENCE_ROOT)")
    d = partfile.read(path, ("pp", "pl"))
    g = np.load(os.path.join(HERE, "golden", "part0104_kat.npz"))
    assert d["np"] == int(g["np_"]) and d["ns"] == int(g["ns"])
    for k in ("mass", "pos", "vel", "ep", "ev", "cpos"):
        assert np.array_equal(d[k], g[k]), k
    for k, cap in (("pp", 12), ("pl", 3)):
        cnt = d[k + "_count"]
        assert np.array_equal(cnt, g[k + "_count"])
        mask = np.arange(cap)[None, :] < cnt[:, None]
        assert np.array_equal(np.where(mask, d[k + "_id"].reshape(-1, cap), 0).ravel(), g[k + "_id"])


def test_part_entry_points_check_arguments():
    from xdynamics_dll_gb300 import _lib
    L = _lib.lib()
    t = C.c_double()
    assert L.xdem_sim_save_part(None, b"x.bin", 0.0) == T.XDEM_ERR_ARG
    assert L.xdem_sim_load_part(None, b"x.bin", C.byref(t)) == T.XDEM_ERR_ARG
