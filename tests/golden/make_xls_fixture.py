"""Writes tests/golden/xls_cube_particle_cells.json: the cells of the
reference workbook resource/cube_particle/cube_particle.xls as read by
xdynamics_dll_gb300.xls.read_cells, so the GPU test that steps a scene
built from a workbook runs where the reference tree is absent.  Run where
the reference sits beside this repository (or set XDEM_REFERENCE_ROOT)."""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from xdynamics_dll_gb300 import xls  # noqa: E402

REF_ROOT = os.environ.get("XDEM_REFERENCE_ROOT") or os.path.join(os.path.dirname(ROOT), "reference")

if __name__ == "__main__":
    src = os.path.join(REF_ROOT, "resource", "cube_particle", "cube_particle.xls")
    cells = xls.read_cells(src)
    out = {"source": "resource/cube_particle/cube_particle.xls",
           "cells": [[r, c, v] for (r, c), v in sorted(cells.items())]}
    with open(os.path.join(HERE, "xls_cube_particle_cells.json"), "w") as f:
        json.dump(out, f, indent=0)
    print(len(cells), "cells")
