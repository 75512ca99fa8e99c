"""Generates the golden fixtures of tests/golden/ (run once where the
reference sources are present; the fixtures are committed).

  part0104_kat.npz  state and pair lists of resource/input/part0104.bin, a
                    snapshot the reference's GPU path wrote (cluster bed of
                    10,584 spheres in 2,646 four-sphere clusters inside a
                    cube).  Pair lists are the known answer for hash -> stable
                    sort -> cluster contact -> cluster plane contact.
  ref_sphere.npz    a dense sphere scene with five planes and a triangle mesh:
                    inputs of one step and the outputs of the reference's own
                    kernels (oracle/_ref) for every launcher of the step.
  ref_cluster.npz   the same for a three-sphere cluster bed with planes and a
                    mesh.
  ref_cylinder.npz  one launch of the reference's particle-cylinder kernels
                    (spheres and cluster members, four material cases).

Usage:  make -C oracle all ref && python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import pyoracle  # noqa: E402
import kseq  # noqa: E402
from xdynamics_dll_gb300 import scenes, types as T  # noqa: E402

# the reference checkout sits beside this repository unless XDEM_REFERENCE_ROOT says otherwise
REF_ROOT = os.environ.get("XDEM_REFERENCE_ROOT") or os.path.join(os.path.dirname(ROOT), "reference")


def read_part_file(path):
    """Part-file layout of xResultManager::export_step_data_to_file
    (source/xdynamics_manager/xResultManager.cpp:828-903), version 2, with
    particle-particle and particle-plane blocks."""
    b = open(path, "rb").read()
    off = [0]

    def take(dt, n):
        a = np.frombuffer(b, dtype=dt, count=n, offset=off[0]).copy()
        off[0] += a.nbytes
        return a
    d = {}
    d["ct"] = take("<f8", 1)[0]
    npart, ncl = (int(x) for x in take("<u4", 2))
    d["np"], d["ns"] = npart, ncl
    d["mass"] = take("<f8", ncl)
    d["pos"] = take("<f8", npart * 4)
    d["vel"] = take("<f8", ncl * 3)
    d["acc"] = take("<f8", ncl * 3)
    d["ep"] = take("<f8", ncl * 4)
    d["ev"] = take("<f8", ncl * 4)
    d["ea"] = take("<f8", ncl * 4)
    if npart != ncl:
        d["cpos"] = take("<f8", ncl * 4)
    d["pp_count"] = take("<u4", npart)
    d["pp_id"] = take("<u4", npart * T.MAX_P2P_COUNT)
    d["pp_tsd"] = take("<f8", npart * T.MAX_P2P_COUNT * 2)
    d["pl_count"] = take("<u4", npart)
    d["pl_id"] = take("<u4", npart * T.MAX_P2PL_COUNT)
    d["pl_tsd"] = take("<f8", npart * T.MAX_P2PL_COUNT * 2)
    assert off[0] == len(b), (off[0], len(b))
    return d


def make_kat():
    d = read_part_file(os.path.join(REF_ROOT, "resource", "input", "part0104.bin"))
    n = d["np"]
    # keep only the stored slots of the pair lists
    pp_mask = (np.arange(T.MAX_P2P_COUNT)[None, :] < d["pp_count"][:, None]).ravel()
    pl_mask = (np.arange(T.MAX_P2PL_COUNT)[None, :] < d["pl_count"][:, None]).ravel()
    np.savez_compressed(
        os.path.join(HERE, "part0104_kat.npz"),
        ct=d["ct"], np_=n, ns=d["ns"], mass=d["mass"], pos=d["pos"], vel=d["vel"], ep=d["ep"], ev=d["ev"],
        cpos=d["cpos"], pp_count=d["pp_count"], pp_id=np.where(pp_mask, d["pp_id"], 0).astype(np.uint32),
        pl_count=d["pl_count"], pl_id=np.where(pl_mask, d["pl_id"], 0).astype(np.uint32),
        # scene of the snapshot: resource/WheelTestBedWithCluster/
        # Wheeltestbedcluster_drive_JJS(14_0.2_3).xls cube, grid of
        # xDiscreteElementMethodSimulation.cpp:94-102
        cube_min=np.array([-1.045, -0.1, -0.130]), cube_max=np.array([-0.345, 0.4, 0.130]),
        cell_size=0.01, xci=np.array([0, 0, d["ns"], 4], dtype=np.uint32))


def sphere_scene():
    sc = scenes.random_packed(700, 0.8e-3, 1.2e-3, None, seed=11, rfric=0.05, cell_factor=2.0)
    # a small closed mesh (uv sphere) pushed into the packing
    mesh = scenes.uv_sphere_mesh(2.5e-3, 6, 10)
    pos = sc.pos.reshape(-1, 4)
    c = pos[:, :3].mean(0) + np.array([0.0, 0.0, 0.0])
    body = T.body_record(mass=0.05, pos=c, vel=(0.01, -0.02, 0.0), ep=(1.0, 0.0, 0.0, 0.0),
                         ed=(0.0, 0.3, 0.1, -0.2))
    sc.meshes = [dict(vlist_local=mesh, body=body, cp=sc.pp_cp)]
    # cell size must cover the largest triangle sphere as well
    return sc


def cluster_scene():
    sc = scenes.cluster_bed(240, neach=3, sub_r=1e-3, seed=5, trough=(0.024, 0.02, 0.024), vel_scale=0.02,
                            spacing_factor=0.5)
    # walls and floor cut 0.3 mm into the bed so boundary spheres touch them
    sc.planes = scenes.open_box_planes(3e-4, 0.024 - 3e-4, 3e-4, 0.03, 3e-4, 0.024 - 3e-4)
    mesh = scenes.uv_sphere_mesh(2.0e-3, 6, 8)
    cpos = sc.cpos.reshape(-1, 4)
    c = cpos[:, :3].mean(0)
    body = T.body_record(mass=0.02, pos=c, vel=(0.0, 0.0, 0.01), ep=(1.0, 0.0, 0.0, 0.0),
                         ed=(0.0, 0.0, 0.2, 0.0))
    sc.meshes = [dict(vlist_local=mesh, body=body, cp=sc.pp_cp)]
    return sc


def fit_cell(sc, meshes):
    rmax = max(float(sc.pos.reshape(-1, 4)[:, 3].max()),
               max((float(m["sphere"].reshape(-1, 4)[:, 3].max()) for m in meshes), default=0.0))
    sc.cell_size = 2.0 * rmax


def struct_bytes(s):
    import ctypes as C
    return np.frombuffer(C.string_at(C.addressof(s), C.sizeof(s)), dtype=np.uint8).copy()


def run_ref_pair(sc, kind):
    O = pyoracle.Oracle()
    R = kseq.RefBackend(pyoracle.RefKernels())
    meshes = kseq.mesh_arrays(sc, O)
    fit_cell(sc, meshes)
    s = kseq.state_arrays(sc)
    # warm-up step fills the pair lists (history), then the recorded step
    step = kseq.sphere_step if kind == "sphere" else kseq.cluster_step
    if kind == "sphere":
        step(R, sc, s, meshes, compat=1)
    else:
        step(R, sc, s, meshes)
    inputs = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in s.items() if k != "bf"}
    if kind == "sphere":
        g, _, partials = step(R, sc, s, meshes, compat=1)
    else:
        g, _, partials = step(R, sc, s, meshes)
    out = {}
    for k, v in inputs.items():
        if isinstance(v, np.ndarray):
            out["in_" + k] = v
    for k in kseq.OUT_KEYS + (["cpos"] if kind == "cluster" else []):
        out["out_" + k] = s[k]
    for k in ("hash", "index", "sorted_index"):
        out["out_" + k] = g[k]
    occ = g["cstart"] != 0xFFFFFFFF
    out["out_cells"] = np.nonzero(occ)[0].astype(np.uint32)
    out["out_cstart"] = g["cstart"][occ]
    out["out_cend"] = g["cend"][occ]
    out["out_partials"] = np.array([np.stack(p) for p in partials])
    out["prm"] = struct_bytes(sc.params())
    out["planes"] = np.stack([struct_bytes(p) for p in sc.planes])
    out["plane_body"] = np.stack(sc.plane_body)
    out["pp_cp"] = struct_bytes(sc.pp_cp)
    m = meshes[0]
    out["mesh_dti"] = np.frombuffer(bytes(m["dti"]), dtype=np.uint8).copy()
    out["mesh_sphere"] = m["sphere"]
    out["mesh_dlocal"] = m["dlocal"]
    out["mesh_vlist"] = m["vlist"]
    out["mesh_body"] = m["body"]
    out["ntri"] = m["ntri"]
    np.savez_compressed(os.path.join(HERE, f"ref_{kind}.npz"), **out)


def make_cylinder():
    """ref_cylinder.npz: one launch of the reference's cylinder kernels
    (cylinder_contact_force_kernel / cluster_cylinder_contact_force_kernel,
    impl:1324-1601) for spheres and for cluster members, with Hertz-Mindlin
    and DHS, rolling friction and cohesion, on the seeded inputs of
    kseq.cylinder_inputs (every detection region); inputs and outputs."""
    ref = pyoracle.RefKernels()
    out = {}
    for ci, cluster in enumerate((False, True)):
        for mi, (model, rf, coh) in enumerate(kseq.CYLINDER_CASES):
            inp = kseq.cylinder_inputs(3 + model, cluster=cluster, n_per=24)
            cp = scenes.default_material(rfric=rf)
            cp.coh = coh

            def run(prm, cyl, body, cp, bf, st, pr):
                ref.set_params(prm)
                n = len(st["pos"]) // 4
                if st["cpos"] is None:
                    ref.cylinder(cyl, body, *bf, st["pos"], st["ep"], st["vel"], st["ev"], st["force"],
                                 st["moment"], cp, st["mass"], st["tmax"], st["rres"], pr["pair_count"],
                                 pr["pair_id"], pr["tsd"], n)
                else:
                    ref.cluster_cylinder(cyl, body, *bf, st["pos"], st["cpos"], st["ep"], st["vel"], st["ev"],
                                         st["force"], st["moment"], st["xci"], cp, st["mass"], st["tmax"],
                                         st["rres"], pr["pair_count"], pr["pair_id"], pr["tsd"], n)
                return 0

            res, _ = kseq.run_cylinder(run, inp, cp, model)
            key = f"c{ci}m{mi}_"
            for k in ("pos", "vel", "ep", "ev", "mass", "pair_count", "pair_id", "tsd", "body"):
                out[key + "in_" + k] = inp[k]
            if cluster:
                out[key + "in_cpos"] = inp["cpos"]
                out[key + "in_xci"] = inp["xci"]
            out[key + "cyl"] = struct_bytes(inp["cyl"])
            out[key + "cp"] = struct_bytes(cp)
            out[key + "model"] = np.array(model)
            for k, v in res.items():
                out[key + "out_" + k] = v
    np.savez_compressed(os.path.join(HERE, "ref_cylinder.npz"), **out)


def main():
    make_kat()
    run_ref_pair(sphere_scene(), "sphere")
    run_ref_pair(cluster_scene(), "cluster")
    make_cylinder()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
