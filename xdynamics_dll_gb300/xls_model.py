"""xdynamics model workbooks (.xls) to scenes.

read_model(path) follows xDynamicsManager::OpenModelXLS
(source/xdynamics_manager/xDynamicsManager.cpp:158-287): row 0 of sheet 0
holds, from column 2 on, pairs (section name, "row,col" of its first cell,
one-based).  Each section is read as the reference's xXLSReader reads it
(source/xXLSReader.cpp), row by row until a row's first cell is empty:

  SHAPE       name, type, material, then per type (ReadShapeObject :755-860):
              cube (2): two corners; plane (3): four points; cylinder (27):
              length, top and bottom radius, thickness, base and top centres,
              open part; cluster (28): count, radius, "row,col" of the member
              offsets; mesh (19): location, refinement size, STL path; then an
              optional constant velocity "vx,vy,vz" and stop condition
  PARTICLE    name, type, material (not for clusters), then per type
              (ReadDEMParticle :558-700): cube fill (2): dimension, location,
              min and max radius; cluster (28): "cmf", material, location,
              file -- or a cluster shape's name, location, grid, random flag;
              list (99): count and a text file of "x y z r m" lines
  CONTACT     name, model (0 DHS, 1 Hertz-Mindlin), object0, object1, rest,
              stiffness ratio, static and dynamic friction, cohesion,
              rolling factor (ReadContact :722-753, ReadContactData :219-229)
  SIMULATION  device, time step, save step, end time (:905-920)
  GRAVITY     "gx, gy, gz" (:922-941)
  INTEGRATOR  solver name and type pairs (:862-903)
  MASS, JOINT the rows as read (the multibody part, kept raw)

A cell of the wrong kind raises XlsModelError naming the cell, where the
reference's ReadStr / ReadNum throw (:943-985); workbooks of older layouts
(four or five contact numbers where ReadContactData reads six) are refused
as the reference refuses them.

scene_from_model builds a Scene of the DEM part: planes from PLANE and
CUBE shapes (the cube's six planes of xCubeObject::define), cylinders, STL
meshes, materials from the reference's table (GetMaterialConstant,
include/xTypes.h:404-420), the contact properties of the CONTACT rows,
gravity and time step, and the particles of cube fills and list files.
Deterministic rows come out as the reference makes them.  The cube fill's
jitter and a radius range draw on the C library's rand() in the reference
(frand, xAlgebraMath.h:8), which this build cannot replay, so those draws
come from a seeded generator here with the same lattice and ranges.  .cmf
cluster files and the other particle generators raise XlsModelError naming
the row.
"""
import os

import numpy as np

from . import scenes, types as T
from .xls import read_cells

# xShapeType (include/xTypes.h:143-163)
CUBE, PLANE, LINE, MESH, CIRCLE, CYLINDER, CLUSTER = 2, 3, 5, 19, 23, 27, 28
NO_SHAPE_AND_MASS, NO_SHAPE_AND_LIST = 98, 99

# GetMaterialConstant (include/xTypes.h:9-47, 404-420): density, Young's
# modulus, Poisson's ratio, shear modulus, by xMaterialType
# (include/xTypes.h:62-77).  A material outside the table reads as zeros,
# as there.
MATERIALS = {
    1: (7850.0, 2e11, 0.3, 79.3e9),       # steel
    2: (1900.0, 35e6, 0.45, 0.0),         # medium clay
    3: (950.0, 1.1e9, 0.42, 0.0),         # polyethylene
    4: (2180.0, 6.8e10, 0.19, 0.0),       # glass
    5: (1185.0, 3.2e9, 0.37, 0.0),        # acrylic
    6: (2700.0, 70.0e9, 0.34, 0.0),       # aluminum
    7: (2600.0, 4.0e7, 0.3, 0.0),         # sand
    8: (1000.0, 0.0, 0.0, 0.0),           # fluid
}

SECTIONS = ("SHAPE", "MASS", "JOINT", "FORCE", "PARTICLE", "CONTACT", "KERNE", "INTEGRATOR", "SIMULATION",
            "GRAVITY")


class XlsModelError(ValueError):
    pass


def material(mt):
    return MATERIALS.get(int(mt), (0.0, 0.0, 0.0, 0.0))


class _Sheet:
    def __init__(self, cells):
        self.cells = cells

    def empty(self, r, c):
        v = self.cells.get((r, c))
        return v is None or v == ""

    def str(self, r, c):
        v = self.cells.get((r, c))
        if not isinstance(v, str):
            raise XlsModelError(f"Cell[{r}, {c}] is not string type.")
        return v

    def num(self, r, c):
        v = self.cells.get((r, c))
        if not isinstance(v, float):
            raise XlsModelError(f"Cell[{r}, {c}] is not number type.")
        return v

    def vec(self, r, c, n=3, typ=float):
        """A "a, b, c" cell (xstring::split), missing entries 0."""
        out = []
        for p in self.str(r, c).split(",")[:n]:
            p = p.strip()
            try:
                out.append(typ(float(p)) if p else typ(0))
            except ValueError:
                raise XlsModelError(f"Cell[{r}, {c}] does not hold {n} numbers: {self.cells[(r, c)]!r}")
        while len(out) < n:
            out.append(typ(0))
        return out


def _rc(s):
    try:
        r, c = (int(float(x)) for x in s.split(",")[:2])
    except ValueError:
        raise XlsModelError(f"{s!r} is not a row,column pair")
    return r - 1, c - 1


def read_model(path):
    """The workbook's sections as dicts and lists (see the module text)."""
    return model_from_cells(read_cells(path), path)


def model_from_cells(cells, path=""):
    """read_model over cells already read ({(row, col): str or float})."""
    sh = _Sheet(cells)
    model = {"name": sh.cells.get((0, 1), ""), "path": path}
    index = {}
    c = 2
    while not sh.empty(0, c):
        tn = sh.str(0, c)
        loc = sh.str(0, c + 1)
        c += 2
        if tn in SECTIONS:
            index[tn] = _rc(loc)
    for tn, (r, cc) in index.items():
        if sh.empty(r, cc):
            raise XlsModelError(f"Exception in excel reader : Information cell[{r}, {cc}] of {tn} is empty.")
    model["index"] = index
    if "SHAPE" in index:
        model["shapes"] = _shapes(sh, *index["SHAPE"])
    if "PARTICLE" in index:
        model["particles"] = _particles(sh, *index["PARTICLE"])
    if "CONTACT" in index:
        model["contacts"] = _contacts(sh, *index["CONTACT"])
    if "SIMULATION" in index:
        r, cc = index["SIMULATION"]
        sim = {}
        for key, conv in (("device", sh.str), ("dt", sh.num), ("save_step", sh.num), ("end_time", sh.num)):
            if sh.empty(r, cc):
                break
            sim[key] = conv(r, cc)
            cc += 1
        model["simulation"] = sim
    if "GRAVITY" in index:
        r, cc = index["GRAVITY"]
        if not sh.empty(r, cc):
            model["gravity"] = tuple(sh.vec(r, cc))
    if "INTEGRATOR" in index:
        r, cc = index["INTEGRATOR"]
        integ = {}
        while not sh.empty(r, cc):
            integ[sh.str(r, cc)] = int(sh.num(r, cc + 1))
            r += 1
        model["integrator"] = integ
    for tn in ("MASS", "JOINT"):
        if tn in index:
            r, cc = index[tn]
            rows = []
            while not sh.empty(r, cc):
                row = []
                k = cc
                while not sh.empty(r, k):
                    row.append(sh.cells[(r, k)])
                    k += 1
                rows.append(row)
                r += 1
            model[tn.lower()] = rows
    return model


def _shapes(sh, r, c0):
    out = []
    while not sh.empty(r, c0):
        c = c0
        name = sh.str(r, c); c += 1
        form = int(sh.num(r, c)); c += 1
        mat = int(sh.num(r, c)); c += 1
        d = {"name": name, "type": form, "material": mat}
        if form == CUBE:
            d["p0"] = sh.vec(r, c); d["p1"] = sh.vec(r, c + 1); c += 2
        elif form == LINE:
            d["points"] = [sh.vec(r, c + k) for k in range(3)]; c += 3
        elif form == PLANE:
            d["points"] = [sh.vec(r, c + k) for k in range(4)]; c += 4
        elif form == CYLINDER:
            d["length"], d["r_top"], d["r_bottom"], d["thickness"] = (sh.num(r, c + k) for k in range(4)); c += 4
            d["p0"] = sh.vec(r, c); d["p1"] = sh.vec(r, c + 1); c += 2
            # the open part (ReadCylinderObjectData :231-264; values of
            # xCylinderObject::empty_part)
            ep = sh.str(r, c); c += 1
            parts = {"noempty": 0, "top": 1, "bottom": 2, "radial": 4}
            if ep not in parts:
                raise XlsModelError(f"Unsupported cylinder[{name}] empty information.")
            d["empty_part"] = parts[ep]
        elif form == CLUSTER:
            num = int(sh.num(r, c)); c += 1
            rad = sh.num(r, c); c += 1
            lr, lc = _rc(sh.str(r, c)); c += 1
            d["count"], d["radius"] = num, rad
            d["rloc"] = [sh.vec(lr, lc + k) for k in range(num)]
        elif form == MESH:
            d["location"] = sh.vec(r, c); c += 1
            d["refinement"] = sh.num(r, c); c += 1
            d["file"] = sh.str(r, c); c += 1
        else:
            raise XlsModelError(f"Unsupported shape[{name}] type.")
        if not sh.empty(r, c):
            d["moving_velocity"] = sh.vec(r, c); c += 1
            if not sh.empty(r, c):
                d["stop_condition"] = sh.str(r, c); c += 1
        out.append(d)
        r += 1
    return out


def _particles(sh, r, c0):
    out = []
    while not sh.empty(r, c0):
        c = c0
        name = sh.str(r, c); c += 1
        form = int(sh.num(r, c)); c += 1
        d = {"name": name, "type": form}
        if form != CLUSTER:
            d["material"] = int(sh.num(r, c)); c += 1
        if form == CUBE:
            d["dimension"] = sh.vec(r, c); d["location"] = sh.vec(r, c + 1); c += 2
            d["min_radius"], d["max_radius"] = sh.num(r, c), sh.num(r, c + 1); c += 2
        elif form == CLUSTER:
            obj = sh.str(r, c); c += 1
            if obj == "cmf":
                d["source"] = "cmf"
                d["material"] = int(sh.num(r, c)); c += 1
                d["location"] = sh.vec(r, c); c += 1
                d["file"] = sh.str(r, c); c += 1
            else:
                d["source"] = obj
                d["location"] = sh.vec(r, c); c += 1
                d["grid"] = sh.vec(r, c, typ=int); c += 1
                d["random"] = sh.str(r, c) == "true"; c += 1
        elif form == NO_SHAPE_AND_LIST:
            d["count"] = int(sh.num(r, c)); c += 1
            d["file"] = sh.str(r, c); c += 1
        elif form == NO_SHAPE_AND_MASS:
            d["radius"] = sh.num(r, c); c += 1
        else:
            d["fields"] = []
            while not sh.empty(r, c):
                d["fields"].append(sh.cells[(r, c)])
                c += 1
        if not sh.empty(r, c):
            d["extra"] = sh.cells[(r, c)]
        out.append(d)
        r += 1
    return out


def _contacts(sh, r, c0):
    out = []
    while not sh.empty(r, c0):
        c = c0
        d = {"name": sh.str(r, c), "model": int(sh.num(r, c + 1)), "object0": sh.str(r, c + 2),
             "object1": sh.str(r, c + 3)}
        c += 4
        for key in ("rest", "rto", "mu_s", "mu", "coh", "rf"):
            d[key] = sh.num(r, c)
            c += 1
        out.append(d)
        r += 1
    return out


def cube_fill(d, rng):
    """CreateCubeParticle (xParticleManager.cpp:646-700): a lattice of
    spheres of radius max_radius filling the box of `dimension` at
    `location`, each centre moved by U[0, 1) times r * (spacing slack) on
    every axis, radii U[min, max] when they differ (the U[0, 1) draws from
    `rng` stand in for the reference's frand())."""
    dx, dy, dz = d["dimension"]
    lx, ly, lz = d["location"]
    r = d["max_radius"]
    dia = 2.0 * r
    nd = np.array([int(dx / dia) - 1, int(dy / dia) - 1, int(dz / dia) - 1])
    if np.any(nd <= 0):
        return np.zeros((0, 4))
    space = (np.array([dx, dy, dz]) - dia * nd) / (nd + 1)
    gab = dia + space
    ran = r * space
    pts = []
    for z in range(nd[2]):
        for y in range(nd[1]):
            for x in range(nd[0]):
                u = rng.random(3)
                pts.append((lx + r + space[0] + x * gab[0] + ran[0] * u[0],
                            ly + r + space[1] + y * gab[1] + ran[1] * u[1],
                            lz + r + space[2] + z * gab[2] + ran[2] * u[2], r))
    pos = np.array(pts, dtype=np.float64)
    if d["min_radius"] != d["max_radius"]:
        pos[:, 3] = d["min_radius"] + (d["max_radius"] - d["min_radius"]) * rng.random(len(pos))
    return pos


def find_file(path, search):
    """A file the workbook names, often by a Windows path of the machine it
    was written on: the path itself, else its file name in each directory
    of `search`."""
    if os.path.exists(path):
        return path
    base = path.replace("\\", "/").split("/")[-1]
    for d in search:
        if d and os.path.exists(os.path.join(d, base)):
            return os.path.join(d, base)
    return None


def read_stl_ascii(path, scale=0.001):
    """Triangles [ntri, 9] of an ASCII STL, scaled from millimetres to
    metres as xMeshObject::DefineShapeFromFile does (xMeshObject.cpp:61-128:
    three header words, then per facet its normal and three vertices)."""
    tris, cur = [], []
    for line in open(path, errors="replace"):
        w = line.split()
        if len(w) == 4 and w[0] == "vertex":
            cur += [scale * float(x) for x in w[1:]]
            if len(cur) == 9:
                tris.append(cur)
                cur = []
    return np.asarray(tris, dtype=np.float64).reshape(-1, 9)


def _contact_property(c, mat0, mat1):
    rho0, E0, nu0, G0 = material(mat0)
    rho1, E1, nu1, G1 = material(mat1)
    # device_contact_property in the order of xContact::define
    # (xContact.cpp:304-312): Ei, Ej, pri, prj, Gi, Gj, rest, fric, s_fric,
    # rfric, coh, sratio, amp
    return T.ContactProperty(E0, E1, nu0, nu1, G0, G1, c["rest"], c["mu"], c["mu_s"], c["rf"], c["coh"], c["rto"],
                             1.0)


def scene_from_model(model, seed=0, base_dir=None, cell_factor=2.0):
    """The DEM scene of a model read by read_model (see the module text).
    Files the workbook names (particle lists, STL meshes) are looked up as
    find_file does, in the workbook's directory and base_dir."""
    rng = np.random.default_rng(seed)
    search = [os.path.dirname(model.get("path", "")), base_dir]
    shapes = {s["name"]: s for s in model.get("shapes", [])}
    mats = {n: s["material"] for n, s in shapes.items()}
    pos_parts, mass_parts = [], []
    pnames = [p["name"] for p in model.get("particles", [])]
    for p in model.get("particles", []):
        mats[p["name"]] = p.get("material", 0)
        if p["type"] == CUBE:
            pos = cube_fill(p, rng)
            rho = material(p["material"])[0]
            pos_parts.append(pos)
            mass_parts.append(rho * (4.0 / 3.0) * np.pi * pos[:, 3] ** 3)
        elif p["type"] == NO_SHAPE_AND_LIST:
            f = find_file(p["file"], search)
            if not f:
                raise XlsModelError(f"particle list {p['file']} of row {p['name']} not found")
            a = np.loadtxt(f, ndmin=2)[:p["count"]]
            pos_parts.append(a[:, :4])
            mass_parts.append(a[:, 4])
        else:
            raise XlsModelError(f"particle row {p['name']}: source type {p['type']} needs files or draws this "
                                "build does not reproduce (cluster .cmf, plane/line/circle fills)")
    if not pos_parts:
        raise XlsModelError("model has no particles")
    pos = np.concatenate(pos_parts)
    mass = np.concatenate(mass_parts)
    n = pos.shape[0]
    J = (2.0 / 5.0) * mass * pos[:, 3] ** 2
    vel, acc, ep, ev, ea = scenes._init_state(n)
    g = tuple(model.get("gravity", (0.0, scenes.G_Y, 0.0)))
    acc = np.zeros(n * 3)
    acc[0::3], acc[1::3], acc[2::3] = g
    planes, plane_cp, cylinders, meshes = [], [], [], []
    pp_cp, cmodel = None, 1
    for c in model.get("contacts", []):
        o0, o1 = c["object0"], c["object1"]
        cp = _contact_property(c, mats.get(o0, 0), mats.get(o1, 0))
        if o0 == o1:
            pp_cp, cmodel = cp, c["model"]
            continue
        other = o1 if o0 in pnames else o0
        s = shapes.get(other)
        if s is None:
            raise XlsModelError(f"contact {c['name']} names {other}, which is no shape")
        if s["type"] == CUBE:
            new = T.cube_planes(s["p0"], s["p1"], first_id=len(planes))
        elif s["type"] == PLANE:
            pts = s["points"]
            # xPlaneObject::define(p0, p1, p2, p3) (xPlaneObject.cpp:22-43):
            # xw = p0, w2 = p1, w4 = p3
            new = [T.plane_from_points(len(planes), pts[0], pts[1], pts[3])]
        elif s["type"] == CYLINDER:
            # xCylinderObject::SetupDataFromStructure (xCylinderObject.cpp:
            # 78-108): the body at the midpoint, both ends in its frame
            pb, pt = np.asarray(s["p0"], float), np.asarray(s["p1"], float)
            mid = 0.5 * (pb + pt)
            cyl = T.CylinderInfo()
            cyl.id = len(cylinders)
            cyl.empty_part = s["empty_part"]
            cyl.thickness = s["thickness"]
            cyl.len_rr = T.Double3(s["length"], s["r_top"], s["r_bottom"])
            cyl.pbase = T.Double3(*(pb - mid))
            cyl.ptop = T.Double3(*(pt - mid))
            cylinders.append(dict(cyl=cyl, body=T.body_record(pos=mid), cp=cp))
            continue
        elif s["type"] == MESH:
            f = find_file(s["file"], search)
            if not f:
                raise XlsModelError(f"mesh file {s['file']} of shape {s['name']} not found")
            tris = read_stl_ascii(f)
            loc = np.asarray(s["location"], float)
            # vertices in the frame of the body at `location`
            meshes.append(dict(vlist_local=tris - np.tile(loc, 3)[None, :], body=T.body_record(pos=loc), cp=cp))
            continue
        else:
            raise XlsModelError(f"contact {c['name']}: shape type {s['type']} is not built from a workbook here")
        planes += new
        plane_cp += [cp] * len(new)
    if pp_cp is None:
        raise XlsModelError("model has no particle-particle contact")
    rmax = float(pos[:, 3].max())
    sim = model.get("simulation", {})
    return scenes.Scene(np_=n, ns=n, pos=pos.ravel(), vel=vel, acc=acc, ep=ep, ev=ev, ea=ea, mass=mass,
                        inertia=np.repeat(J, 3), dt=float(sim.get("dt", 1e-5)), cell_size=cell_factor * rmax,
                        gravity=g, contact_model=cmodel, pp_cp=pp_cp, planes=planes, plane_cp=plane_cp,
                        plane_body=[T.body_record() for _ in planes], cylinders=cylinders, meshes=meshes,
                        name=str(model.get("name", "")),
                        note=f"{n} spheres from {os.path.basename(model.get('path', ''))}")
