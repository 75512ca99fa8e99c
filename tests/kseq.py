"""Kernel sequences run through interchangeable back ends.

A back end is the C oracle (oracle/pyoracle.Oracle), the reference's own
kernels compiled for the host (oracle/pyoracle.RefKernels) or the GPU library
(xdynamics_dll_gb300.launchers.Launchers).  Each sequence takes a scene
(xdynamics_dll_gb300.scenes.Scene), runs one pass of the reference's
launchers in the order of xIntegratorVV::OneStepSimulation on copies of its
arrays and returns every output array by name.
"""
import numpy as np

from xdynamics_dll_gb300 import types as T

NCELL_CACHE = {}


def _zeros(n, dt=np.float64):
    return np.zeros(n, dtype=dt)


def grid_arrays(prm, nentry):
    ncell = prm.ncell
    return dict(hash=_zeros(nentry, np.uint32), index=_zeros(nentry, np.uint32),
                cstart=_zeros(ncell, np.uint32), cend=_zeros(ncell, np.uint32),
                sorted_index=_zeros(nentry, np.uint32))


class OracleBackend:
    def __init__(self, oracle):
        self.o = oracle
        self.prm = None

    def set_params(self, prm):
        self.prm = prm

    def vv_pos(self, s):
        self.o.vv_update_position(self.prm, s["pos"], s["ep"], s["vel"], s["ev"], s["acc"], s["ea"], s["np"])

    def vv_vel(self, s, compat):
        self.o.vv_update_velocity(self.prm, s["vel"], s["acc"], s["ep"], s["ev"], s["ea"], s["force"],
                                  s["moment"], s["mass"], s["inertia"], s["np"], compat)

    def hash(self, g, pos, sid, n):
        return self.o.hash(self.prm, g["hash"], g["index"], pos, sid, n)

    def reorder(self, g, n):
        self.o.reorder(g["hash"], g["index"], g["cstart"], g["cend"], g["sorted_index"], n, self.prm.ncell)

    def p2p(self, s, g, cp):
        return self.o.p2p(self.prm, s["pos"], s["ep"], s["vel"], s["ev"], s["force"], s["moment"], s["mass"],
                          s["tmax"], s["rres"], s["pp_count"], s["pp_id"], s["pp_tsd"], g["sorted_index"],
                          g["cstart"], g["cend"], cp, s["np"])

    def plane(self, s, plane, dbi, cp):
        return self.o.plane(self.prm, plane, dbi, cp, s["bf"], s["pos"], s["ep"], s["vel"], s["ev"], s["force"],
                            s["moment"], s["mass"], s["tmax"], s["rres"], s["pl_count"], s["pl_id"], s["pl_tsd"],
                            s["np"])

    def cylinder(self, s, cyl, dbi, cp):
        return self.o.cylinder(self.prm, cyl, dbi, cp, s["bf"], s["pos"], s.get("cpos"), s["ep"], s["vel"],
                               s["ev"], s["force"], s["moment"], s["mass"], s["tmax"], s["rres"], s["cy_count"],
                               s["cy_id"], s["cy_tsd"], s.get("xci"), s["np"])

    def mesh(self, s, g, dti, dbi, cp, ntri):
        return self.o.mesh(self.prm, dti, dbi, s["bf"], s["pos"], s["ep"], s["vel"], s["ev"], s["force"],
                           s["moment"], s["mass"], s["tmax"], s["rres"], s["ms_count"], s["ms_id"], s["ms_tsd"],
                           g["sorted_index"], g["cstart"], g["cend"], cp, s["np"], ntri)

    def rolling(self, s):
        self.o.rolling(self.prm, s["tmax"], s["rres"], s["inertia"], s["ep"], s["ev"], s["moment"], s["np"],
                       s.get("rolling_per_sphere", 0))

    def update_mesh(self, dbi, vlist, sphere, dlocal, dti, ntri):
        self.o.update_mesh(dbi, vlist, sphere, dlocal, dti, ntri)

    def clusters_p2p(self, s, g, cp):
        return self.o.clusters_p2p(self.prm, s["pos"], s["cpos"], s["ep"], s["vel"], s["ev"], s["force"],
                                   s["moment"], s["mass"], s["tmax"], s["rres"], s["pp_count"], s["pp_id"],
                                   s["pp_tsd"], g["sorted_index"], g["cstart"], g["cend"], cp, s["xci"], s["np"])

    def cluster_plane(self, s, plane, dbi, cp):
        return self.o.cluster_plane(self.prm, plane, dbi, s["bf"], s["pos"], s["cpos"], s["ep"], s["vel"],
                                    s["ev"], s["force"], s["moment"], cp, s["mass"], s["tmax"], s["rres"],
                                    s["pl_count"], s["pl_id"], s["pl_tsd"], s["xci"], s["np"])

    def cluster_mesh(self, s, g, dti, dbi, cp, ntri):
        return self.o.cluster_mesh(self.prm, dti, dbi, s["bf"], s["pos"], s["cpos"], s["ep"], s["vel"], s["ev"],
                                   s["force"], s["moment"], cp, s["mass"], s["tmax"], s["rres"], s["ms_count"],
                                   s["ms_id"], s["ms_tsd"], g["sorted_index"], g["cstart"], g["cend"], s["xci"],
                                   s["np"], ntri)

    def cluster_rolling(self, s):
        self.o.cluster_rolling(self.prm, s["tmax"], s["rres"], s["inertia"], s["ep"], s["ev"], s["moment"],
                               s["xci"], s["np"])

    def vv_cluster_pos(self, s):
        self.o.vv_cluster_position(self.prm, s["pos"], s["cpos"], s["ep"], s["rloc"], s["vel"], s["acc"], s["ev"],
                                   s["ea"], s["xci"], s["ns"])

    def vv_cluster_vel(self, s):
        self.o.vv_cluster_velocity(self.prm, s["cpos"], s["ep"], s["vel"], s["acc"], s["ev"], s["ea"], s["force"],
                                   s["moment"], s["rloc"], s["mass"], s["inertia"], s["xci"], s["ns"])


class RefBackend:
    """The reference kernels compiled for the host.  Its sphere velocity
    kernel is the literal reference one (linear velocity unchanged), so
    vv_vel is only comparable with compat=1."""

    def __init__(self, ref):
        self.r = ref

    def set_params(self, prm):
        self.r.set_params(prm)

    def vv_pos(self, s):
        self.r.vv_update_position(s["pos"], s["ep"], s["vel"], s["ev"], s["acc"], s["ea"], s["np"])

    def vv_vel(self, s, compat):
        assert compat == 1
        self.r.vv_update_velocity(s["vel"], s["acc"], s["ep"], s["ev"], s["ea"], s["force"], s["moment"],
                                  s["mass"], s["inertia"], s["np"])

    def hash(self, g, pos, sid, n):
        self.r.hash(g["hash"], g["index"], pos, sid, n)
        return 0

    def reorder(self, g, n):
        self.r.reorder(g["hash"], g["index"], g["cstart"], g["cend"], g["sorted_index"], n, g["cstart"].size)

    def p2p(self, s, g, cp):
        self.r.p2p(s["pos"], s["ep"], s["vel"], s["ev"], s["force"], s["moment"], s["mass"], s["tmax"], s["rres"],
                   s["pp_count"], s["pp_id"], s["pp_tsd"], g["sorted_index"], g["cstart"], g["cend"], cp, s["np"])
        return 0

    def plane(self, s, plane, dbi, cp):
        self.r.plane(plane, dbi, cp, *s["bf"], s["pos"], s["ep"], s["vel"], s["ev"], s["force"], s["moment"],
                     s["mass"], s["tmax"], s["rres"], s["pl_count"], s["pl_id"], s["pl_tsd"], s["np"])
        return 0

    def mesh(self, s, g, dti, dbi, cp, ntri):
        self.r.mesh(dti, dbi, *s["bf"], s["pos"], s["ep"], s["vel"], s["ev"], s["force"], s["moment"], s["mass"],
                    s["tmax"], s["rres"], s["ms_count"], s["ms_id"], s["ms_tsd"], s["dsph"], g["sorted_index"],
                    g["cstart"], g["cend"], cp, s["np"], ntri)
        return 0

    def rolling(self, s):
        self.r.rolling(s["tmax"], s["rres"], s["inertia"], s["ep"], s["ev"], s["moment"], s["np"])

    def update_mesh(self, dbi, vlist, sphere, dlocal, dti, ntri):
        self.r.update_mesh(dbi, vlist, sphere, dlocal, dti, ntri)

    def clusters_p2p(self, s, g, cp):
        self.r.clusters_p2p(s["pos"], s["cpos"], s["ep"], s["vel"], s["ev"], s["force"], s["moment"], s["mass"],
                            s["tmax"], s["rres"], s["pp_count"], s["pp_id"], s["pp_tsd"], g["sorted_index"],
                            g["cstart"], g["cend"], cp, s["xci"], s["np"])
        return 0

    def cluster_plane(self, s, plane, dbi, cp):
        self.r.cluster_plane(plane, dbi, *s["bf"], s["pos"], s["cpos"], s["ep"], s["vel"], s["ev"], s["force"],
                             s["moment"], cp, s["mass"], s["tmax"], s["rres"], s["pl_count"], s["pl_id"],
                             s["pl_tsd"], s["xci"], s["np"])
        return 0

    def cluster_mesh(self, s, g, dti, dbi, cp, ntri):
        self.r.cluster_mesh(dti, dbi, *s["bf"], s["pos"], s["cpos"], s["ep"], s["vel"], s["ev"], s["force"],
                            s["moment"], cp, s["mass"], s["tmax"], s["rres"], s["ms_count"], s["ms_id"],
                            s["ms_tsd"], g["sorted_index"], g["cstart"], g["cend"], s["xci"], s["np"], ntri)
        return 0

    def cluster_rolling(self, s):
        self.r.cluster_rolling(s["tmax"], s["rres"], s["inertia"], s["ep"], s["ev"], s["moment"], s["xci"],
                               s["np"])

    def vv_cluster_pos(self, s):
        self.r.vv_cluster_position(s["pos"], s["cpos"], s["ep"], s["rloc"], s["vel"], s["acc"], s["ev"], s["ea"],
                                   s["xci"], s["ns"])

    def vv_cluster_vel(self, s):
        self.r.vv_cluster_velocity(s["cpos"], s["ep"], s["vel"], s["acc"], s["ev"], s["ea"], s["force"],
                                   s["moment"], s["rloc"], s["mass"], s["inertia"], s["xci"], s["ns"])


def state_arrays(scene, seed=None, history=True):
    """Copies of the scene state plus zeroed force/accumulator arrays and
    pair lists.  With history=True the pair lists are pre-filled by a first
    contact pass (so the sequence exercises history lookup)."""
    n, ns = scene.np_, scene.ns
    s = dict(np=n, ns=ns, pos=scene.pos.copy(), vel=scene.vel.copy(), acc=scene.acc.copy(),
             ep=scene.ep.copy(), ev=scene.ev.copy(), ea=scene.ea.copy(), mass=scene.mass.copy(),
             inertia=scene.inertia.copy(), force=_zeros(n * 3), moment=_zeros(n * 3), tmax=_zeros(n * 3),
             rres=_zeros(n), pp_count=_zeros(n, np.uint32), pp_id=_zeros(n * T.MAX_P2P_COUNT, np.uint32),
             pp_tsd=_zeros(n * T.MAX_P2P_COUNT * 2), pl_count=_zeros(n, np.uint32),
             pl_id=_zeros(n * T.MAX_P2PL_COUNT, np.uint32), pl_tsd=_zeros(n * T.MAX_P2PL_COUNT * 2),
             ms_count=_zeros(n, np.uint32), ms_id=_zeros(n * T.MAX_P2MS_COUNT, np.uint32),
             ms_tsd=_zeros(n * T.MAX_P2MS_COUNT * 2), cy_count=_zeros(n, np.uint32),
             cy_id=_zeros(n * T.MAX_P2CY_COUNT, np.uint32), cy_tsd=_zeros(n * T.MAX_P2CY_COUNT * 2),
             bf=[_zeros(n) for _ in range(6)])
    if scene.cpos is not None:
        s["cpos"] = scene.cpos.copy()
        s["xci"] = scene.xci.copy()
        s["rloc"] = scene.rloc.copy()
    return s


def mesh_arrays(scene, oracle):
    """Triangles and bounding spheres of every mesh of the scene, as
    xParticleMeshObjectContact::define builds them (xParticleMeshObjectContact.
    cpp:77-135): vertices placed by the body pose, spheres from
    FitSphereToTriangle(P, Q, R, 0.8), sphere centres also stored in the body
    frame."""
    out = []
    base = 0
    for m in scene.meshes:
        vl = np.ascontiguousarray(m["vlist_local"], dtype=np.float64).reshape(-1, 9)
        ntri = vl.shape[0]
        body = np.asarray(m["body"], dtype=np.float64)
        p = body[T.PX:T.PZ + 1]
        e = body[T.E0:T.E3 + 1]
        A = rot(e)
        dti = (T.TriangleInfo * ntri)()
        sph = np.zeros(ntri * 4)
        loc = np.zeros(ntri * 3)
        for i in range(ntri):
            P = p + A @ vl[i, 0:3]
            Q = p + A @ vl[i, 3:6]
            R = p + A @ vl[i, 6:9]
            dti[i].id = i
            dti[i].tid = base + i
            dti[i].P = T.d3(P); dti[i].Q = T.d3(Q); dti[i].R = T.d3(R)
            c = oracle.fit_sphere(P, Q, R, 0.8)
            sph[4 * i:4 * i + 4] = c
            loc[3 * i:3 * i + 3] = A.T @ (c[:3] - p)
        out.append(dict(ntri=ntri, dti=dti, sphere=sph, dlocal=loc, vlist=vl.ravel().copy(), body=body.copy(),
                        cp=m["cp"], base=base))
        base += ntri
    return out


def rot(e):
    e0, e1, e2, e3 = e
    return np.array([[2 * (e0 * e0 + e1 * e1 - 0.5), 2 * (e1 * e2 - e0 * e3), 2 * (e1 * e3 + e0 * e2)],
                     [2 * (e1 * e2 + e0 * e3), 2 * (e0 * e0 + e2 * e2 - 0.5), 2 * (e2 * e3 - e0 * e1)],
                     [2 * (e1 * e3 - e0 * e2), 2 * (e2 * e3 + e0 * e1), 2 * (e0 * e0 + e3 * e3 - 0.5)]])


def sphere_step(be, scene, s, meshes=(), compat=1, nplanes=None):
    """One step of the sphere path: position, hash (particles then mesh
    spheres), sort/cell start, p2p, planes in id order, meshes, rolling,
    velocity.  Returns (grid arrays, status bits, per-plane/mesh body
    partial snapshots)."""
    prm = scene.params()
    be.set_params(prm)
    st = 0
    be.vv_pos(s)
    ntot = s["np"] + sum(m["ntri"] for m in meshes)
    g = grid_arrays(prm, ntot)
    st |= be.hash(g, s["pos"], 0, s["np"])
    for m in meshes:
        st |= be.hash(g, m["sphere"], s["np"] + m["base"], m["ntri"])
    be.reorder(g, ntot)
    st |= be.p2p(s, g, scene.pp_cp)
    partials = []
    planes = scene.planes if nplanes is None else scene.planes[:nplanes]
    for k, pl in enumerate(planes):
        st |= be.plane(s, pl, np.asarray(scene.plane_body[k]), scene.plane_cp[k])
        partials.append([b.copy() for b in s["bf"]])
    for cy in getattr(scene, "cylinders", []):
        st |= be.cylinder(s, cy["cyl"], np.asarray(cy["body"]), cy["cp"])
        partials.append([b.copy() for b in s["bf"]])
    for m in meshes:
        s["dsph"] = m["sphere"]
        st |= be.mesh(s, g, m["dti"], m["body"], m["cp"], m["ntri"])
        partials.append([b.copy() for b in s["bf"]])
    be.rolling(s)
    be.vv_vel(s, compat)
    return g, st, partials


def cluster_step(be, scene, s, meshes=()):
    prm = scene.params()
    be.set_params(prm)
    st = 0
    be.vv_cluster_pos(s)
    ntot = s["np"] + sum(m["ntri"] for m in meshes)
    g = grid_arrays(prm, ntot)
    st |= be.hash(g, s["pos"], 0, s["np"])
    for m in meshes:
        st |= be.hash(g, m["sphere"], s["np"] + m["base"], m["ntri"])
    be.reorder(g, ntot)
    st |= be.clusters_p2p(s, g, scene.pp_cp)
    partials = []
    for k, pl in enumerate(scene.planes):
        st |= be.cluster_plane(s, pl, np.asarray(scene.plane_body[k]), scene.plane_cp[k])
        partials.append([b.copy() for b in s["bf"]])
    for cy in getattr(scene, "cylinders", []):
        st |= be.cylinder(s, cy["cyl"], np.asarray(cy["body"]), cy["cp"])
        partials.append([b.copy() for b in s["bf"]])
    for m in meshes:
        st |= be.cluster_mesh(s, g, m["dti"], m["body"], m["cp"], m["ntri"])
        partials.append([b.copy() for b in s["bf"]])
    be.cluster_rolling(s)
    be.vv_cluster_vel(s)
    return g, st, partials


OUT_KEYS = ["pos", "vel", "acc", "ep", "ev", "ea", "force", "moment", "tmax", "rres", "pp_count", "pp_id",
            "pp_tsd", "pl_count", "pl_id", "pl_tsd", "ms_count", "ms_id", "ms_tsd"]


def pairs_equal(count_a, id_a, count_b, id_b, cap):
    """Number of particles whose stored pair count and first `count` ids agree."""
    n = count_a.size
    ok = count_a == count_b
    A = id_a.reshape(n, cap)
    B = id_b.reshape(n, cap)
    idx = np.arange(cap)[None, :]
    mask = idx < count_a[:, None]
    same = np.all((A == B) | ~mask, axis=1)
    return int(np.sum(ok & same))


def masked_tsd(count, tsd, cap):
    """History values of the stored slots only (stale slots zeroed)."""
    n = count.size
    t = tsd.reshape(n, cap, 2).copy()
    mask = np.arange(cap)[None, :] < count[:, None]
    t[~mask] = 0.0
    return t.reshape(-1)


def rel_err(a, b, floor):
    """max |a-b| / max(|b|, floor) elementwise."""
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))) if a.size else 0.0


GOLDEN = __import__("os").path.join(__import__("os").path.dirname(__import__("os").path.abspath(__file__)),
                                    "golden")


def _struct(cls, b):
    return cls.from_buffer_copy(bytes(np.asarray(b, dtype=np.uint8)))


def load_ref_fixture(kind):
    """Scene, input state, meshes and expected outputs of ref_<kind>.npz."""
    import os
    from xdynamics_dll_gb300 import scenes
    d = np.load(os.path.join(GOLDEN, f"ref_{kind}.npz"))
    prm = _struct(T.DemParameters, d["prm"])
    planes = [_struct(T.PlaneInfo, b) for b in d["planes"]]
    cp = _struct(T.ContactProperty, d["pp_cp"])
    n = int(prm.np)
    inp = {k[3:]: d[k].copy() for k in d.files if k.startswith("in_")}
    ns = inp["mass"].size
    sc = scenes.Scene(np_=n, ns=ns, pos=inp["pos"], vel=inp["vel"], acc=inp["acc"], ep=inp["ep"], ev=inp["ev"],
                      ea=inp["ea"], mass=inp["mass"], inertia=inp["inertia"], dt=prm.dt, cell_size=prm.cell_size,
                      grid=(prm.grid_size.x, prm.grid_size.y, prm.grid_size.z),
                      origin=(prm.world_origin.x, prm.world_origin.y, prm.world_origin.z),
                      gravity=(prm.gravity.x, prm.gravity.y, prm.gravity.z), contact_model=prm.contact_model,
                      pp_cp=cp, planes=planes, plane_cp=[cp] * len(planes),
                      plane_body=[d["plane_body"][i].copy() for i in range(len(planes))])
    if "cpos" in inp:
        sc.cpos, sc.xci, sc.rloc = inp["cpos"], inp["xci"], inp["rloc"]
    ntri = int(d["ntri"])
    dti = (T.TriangleInfo * ntri).from_buffer_copy(bytes(d["mesh_dti"]))
    meshes = [dict(ntri=ntri, dti=dti, sphere=d["mesh_sphere"].copy(), dlocal=d["mesh_dlocal"].copy(),
                   vlist=d["mesh_vlist"].copy(), body=d["mesh_body"].copy(), cp=cp, base=0)]
    s = state_arrays(sc)
    for k, v in inp.items():
        if k in s and isinstance(s[k], np.ndarray):
            s[k][...] = v
    exp = {k[4:]: d[k] for k in d.files if k.startswith("out_")}
    return sc, s, meshes, exp


def check_outputs(s, g, exp, *, kind, ftol=1e-12, skip=()):
    """Compares one step's outputs with a fixture: integer arrays (cell ids,
    sort order, pair lists) exactly, floating-point arrays to `ftol`
    relative (with an absolute floor of ftol times the array's scale)."""
    occ = g["cstart"] != 0xFFFFFFFF
    assert np.array_equal(np.nonzero(occ)[0], exp["cells"]), "occupied cells differ"
    assert np.array_equal(g["cstart"][occ], exp["cstart"])
    assert np.array_equal(g["cend"][occ], exp["cend"])
    for k in ("hash", "index", "sorted_index"):
        assert np.array_equal(g[k], exp[k]), k
    for k in ("pp_count", "pp_id", "pl_count", "pl_id", "ms_count", "ms_id"):
        if k in skip:
            continue
        assert np.array_equal(s[k], exp[k]), f"{k}: {np.sum(s[k] != exp[k])} entries differ"
    keys = ["pos", "vel", "acc", "ep", "ev", "ea", "force", "moment", "tmax", "rres", "pp_tsd", "pl_tsd",
            "ms_tsd"] + (["cpos"] if kind == "cluster" else [])
    for k in keys:
        if k in skip:
            continue
        a, b = s[k], exp[k]
        scale = max(float(np.max(np.abs(b))) if b.size else 0.0, 1e-300)
        err = float(np.max(np.abs(a - b))) / scale if b.size else 0.0
        assert err <= ftol, f"{k}: max abs diff {np.max(np.abs(a - b)):.3e} (scale {scale:.3e})"


# ---------------------------------------------------------------- cylinders
# (contact model, rolling friction, cohesion) of the cylinder fixtures
CYLINDER_CASES = [(1, 0.0, 0.0), (0, 0.0, 0.0), (1, 0.2, 0.0), (1, 0.0, 5e4)]


def load_cylinder_fixture():
    """Cases of ref_cylinder.npz: (inputs as cylinder_inputs returns them,
    contact property, contact model, the reference kernels' outputs)."""
    import os
    d = np.load(os.path.join(GOLDEN, "ref_cylinder.npz"))
    cases = []
    for ci in range(2):
        for mi in range(len(CYLINDER_CASES)):
            key = f"c{ci}m{mi}_"
            inp = {k: d[key + "in_" + k].copy() for k in ("pos", "vel", "ep", "ev", "mass", "pair_count",
                                                           "pair_id", "tsd", "body")}
            inp["cpos"] = d[key + "in_cpos"].copy() if ci else None
            inp["xci"] = d[key + "in_xci"].copy() if ci else None
            inp["n"] = inp["pos"].size // 4
            inp["ns"] = inp["mass"].size
            inp["cyl"] = _struct(T.CylinderInfo, d[key + "cyl"])
            cp = _struct(T.ContactProperty, d[key + "cp"])
            exp = {k[len(key) + 4:]: d[k] for k in d.files if k.startswith(key + "out_")}
            cases.append((inp, cp, int(d[key + "model"]), exp))
    return cases


def cylinder_inputs(seed, cluster=False, n_per=48):
    """Inputs of one cylinder launch (impl:1324-1601) whose spheres sit in
    every region of the detection: outside and inside the wall, near the
    inner caps (top open: empty_part 1), in the inner corner of the base
    (wall and cap at once), on the annulus beyond an end, near the rim, and
    far away; a rotated, moving, spinning cylinder body; old
    pair lists holding ids k and k + 1000 with history.  cluster=True makes
    every sphere a member of a three-member cluster whose centre, mass,
    velocity and spin the kernel reads instead."""
    rng = np.random.default_rng(seed)
    L, R, th = 0.04, 0.015, 0.002
    cyl = T.CylinderInfo()
    cyl.id = 0
    cyl.empty_part = 1
    cyl.thickness = th
    cyl.len_rr = T.d3((L, R, R))
    cyl.pbase = T.d3((0.0, -0.5 * L, 0.0))
    cyl.ptop = T.d3((0.0, 0.5 * L, 0.0))
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    body = T.body_record(mass=0.7, pos=(0.01, 0.02, -0.005), vel=(0.01, -0.02, 0.03), ep=tuple(q),
                         ed=tuple(0.5 * rng.normal(size=4)))
    A = rot(q)
    pts, rad = [], []

    def add(rho, y, r):
        ph = rng.uniform(0, 2 * np.pi)
        pts.append(np.array([rho * np.cos(ph), y, rho * np.sin(ph)]))
        rad.append(r)

    for _ in range(n_per):
        r = rng.uniform(1e-3, 2e-3)
        add(R + r * rng.uniform(0.3, 1.3), rng.uniform(-0.5 * L + 2 * r, 0.5 * L - 2 * r), r)   # outside wall
        r = rng.uniform(1e-3, 2e-3)
        add(R - r * rng.uniform(0.2, 1.3), rng.uniform(-0.5 * L + 0.5 * r, 0.5 * L - 0.5 * r), r)  # inside wall
        r = rng.uniform(1e-3, 2e-3)
        add(rng.uniform(0.1 * R, R - 2 * r), rng.choice([-1, 1]) * (0.5 * L - r * rng.uniform(0.3, 1.3)), r)  # caps
        r = rng.uniform(1e-3, 2e-3)
        add(rng.uniform(R + 0.1 * th, R + 0.9 * th), rng.choice([-1, 1]) * (0.5 * L + r * rng.uniform(0.2, 1.2)), r)
        r = rng.uniform(1e-3, 2e-3)
        add(R + th + r * rng.uniform(0.1, 0.9), rng.choice([-1, 1]) * (0.5 * L + r * rng.uniform(0.1, 0.9)), r)
        r = rng.uniform(1e-3, 2e-3)
        add(R - r * rng.uniform(0.3, 0.9), -0.5 * L + r * rng.uniform(0.3, 0.9), r)  # inner base corner: wall + cap
        r = rng.uniform(1e-3, 2e-3)
        add(rng.uniform(0, 0.1), rng.uniform(0.1, 0.2), r)                                       # far
    loc = np.array(pts)
    n = len(rad)
    pos = np.zeros((n, 4))
    pos[:, :3] = body[1:4] + loc @ A.T
    pos[:, 3] = rad
    ns = n // 3 if cluster else n
    if cluster:
        n = 3 * ns
        pos = pos[:n]
    vel = rng.normal(0, 0.05, size=(ns, 3))
    ep = rng.normal(size=(ns, 4))
    ep /= np.linalg.norm(ep, axis=1, keepdims=True)
    ev = rng.normal(0, 2.0, size=(ns, 4))
    mass = rng.uniform(1e-5, 5e-5, size=ns)
    out = dict(cyl=cyl, body=body, pos=pos.ravel().copy(), vel=vel.ravel(), ep=ep.ravel(), ev=ev.ravel(),
               mass=mass, n=n, ns=ns, cpos=None, xci=None)
    if cluster:
        cpos = np.zeros((ns, 4))
        cpos[:, :3] = pos.reshape(ns, 3, 4)[:, 1, :3] + rng.normal(0, 1e-3, size=(ns, 3))
        cpos[:, 3] = pos.reshape(ns, 3, 4)[:, 1, 3]
        out["cpos"] = cpos.ravel()
        out["xci"] = np.array([0, 0, ns, 3], dtype=np.uint32)
    pc = rng.integers(0, 3, size=n).astype(np.uint32)
    pid = np.where(rng.random(n * 3) < 0.5, 0, 1000).astype(np.uint32)
    pid[rng.random(n * 3) < 0.2] = 7
    tsd = rng.normal(0, 1e-5, size=n * 6)
    out.update(pair_count=pc, pair_id=pid, tsd=tsd)
    return out


def cylinder_params(inp, model=1):
    prm = T.make_params(np_=inp["n"], dt=1e-5, cell_size=0.004, contact_model=model,
                        ncluster=inp["ns"] if inp["cpos"] is not None else 0,
                        nco=1 if inp["cpos"] is not None else 0)
    return prm


def run_cylinder(run, inp, cp, model=1):
    """One cylinder launch through `run(prm, cyl, body, cp, bf, state, pairs)`
    on copies of the inputs; returns every output array."""
    n = inp["n"]
    st = {k: inp[k].copy() for k in ("pos", "vel", "ep", "ev", "mass")}
    st["cpos"] = None if inp["cpos"] is None else inp["cpos"].copy()
    st["xci"] = inp["xci"]
    st.update(force=np.full(n * 3, 0.25), moment=np.full(n * 3, -0.5), tmax=np.zeros(n * 3), rres=np.zeros(n))
    pairs = dict(pair_count=inp["pair_count"].copy(), pair_id=inp["pair_id"].copy(), tsd=inp["tsd"].copy())
    bf = [np.full(n, 9.0) for _ in range(6)]
    status = run(cylinder_params(inp, model), inp["cyl"], inp["body"].copy(), cp, bf, st, pairs)
    out = dict(force=st["force"], moment=st["moment"], tmax=st["tmax"], rres=st["rres"], **pairs)
    for i, k in enumerate(("fx", "fy", "fz", "mx", "my", "mz")):
        out[k] = bf[i]
    return out, status
