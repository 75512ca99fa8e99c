"""Part files on the host: the layout xResultManager::export_step_data_to_file
writes (source/xdynamics_manager/xResultManager.cpp:828-903, version 2), read
into and written from dicts of numpy arrays.

    time (f64); np, ns (u32); mass[ns]; pos[np*4]; vel, acc[ns*3];
    ep, ev, ea[ns*4]; cpos[ns*4] (clusters only); then for each contact kind
    present, in the order particle pairs, planes, cylinders, triangles:
    count[np] (u32), id[np*cap] (u32), tsd[np*cap*2] (f64), with cap 12
    (particle pairs), 3 (planes), 3 (cylinders), 5 (triangles).

A file does not say which pair blocks it holds: the reader takes them from
the model (`kinds`), as the reference does, and checks that the sizes add
up.  The multibody block of models with a multibody system is not read.
Handles write and read the same layout with xdem_sim_save_part / load_part.
"""
import numpy as np

CAPS = {"pp": 12, "pl": 3, "cy": 3, "ms": 5}
ORDER = ("pp", "pl", "cy", "ms")


def _ordered(kinds):
    bad = [k for k in kinds if k not in CAPS]
    if bad:
        raise ValueError(f"unknown pair blocks {bad}")
    return [k for k in ORDER if k in kinds]


def read(path, kinds=("pp", "pl")):
    b = open(path, "rb").read()
    off = [0]

    def take(dt, n):
        a = np.frombuffer(b, dtype=dt, count=n, offset=off[0]).copy()
        off[0] += a.nbytes
        return a

    d = {"time": float(take("<f8", 1)[0])}
    npart, ns = (int(x) for x in take("<u4", 2))
    d["np"], d["ns"] = npart, ns
    d["mass"] = take("<f8", ns)
    d["pos"] = take("<f8", npart * 4)
    d["vel"] = take("<f8", ns * 3)
    d["acc"] = take("<f8", ns * 3)
    d["ep"] = take("<f8", ns * 4)
    d["ev"] = take("<f8", ns * 4)
    d["ea"] = take("<f8", ns * 4)
    if npart != ns:
        d["cpos"] = take("<f8", ns * 4)
    for k in _ordered(kinds):
        cap = CAPS[k]
        d[k + "_count"] = take("<u4", npart)
        d[k + "_id"] = take("<u4", npart * cap)
        d[k + "_tsd"] = take("<f8", npart * cap * 2)
    if off[0] != len(b):
        raise ValueError(f"{path}: {len(b) - off[0]} bytes left after the blocks of {kinds}")
    return d


def write(path, d, kinds=("pp", "pl")):
    npart, ns = int(d["np"]), int(d["ns"])
    with open(path, "wb") as f:
        f.write(np.asarray([d.get("time", 0.0)], "<f8").tobytes())
        f.write(np.asarray([npart, ns], "<u4").tobytes())
        for k, n in (("mass", ns), ("pos", npart * 4), ("vel", ns * 3), ("acc", ns * 3), ("ep", ns * 4),
                     ("ev", ns * 4), ("ea", ns * 4)):
            a = np.asarray(d[k], "<f8").ravel()
            if a.size != n:
                raise ValueError(f"{k}: {a.size} values, {n} expected")
            f.write(a.tobytes())
        if npart != ns:
            f.write(np.asarray(d["cpos"], "<f8").ravel().tobytes())
        for k in _ordered(kinds):
            cap = CAPS[k]
            f.write(np.asarray(d[k + "_count"], "<u4").ravel().tobytes())
            f.write(np.asarray(d[k + "_id"], "<u4").ravel().tobytes())
            a = np.asarray(d[k + "_tsd"], "<f8").ravel()
            if a.size != npart * cap * 2:
                raise ValueError(f"{k}_tsd: {a.size} values")
            f.write(a.tobytes())
