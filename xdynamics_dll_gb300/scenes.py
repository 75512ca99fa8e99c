"""Synthetic DEM scenes in the reference layout (host numpy arrays).

Mass and inertia follow xParticleManager::SetMassAndInertia
(source/xdynamics_manager/xParticleManager.cpp:1124-1140: m = rho 4/3 pi r^3,
J = 2/5 m r^2 on each axis) and, for clusters, SetClusterMassAndInertia
(:1058-1101).  Initial state follows xDiscreteElementMethodSimulation::
Initialize (source/xdynamics_simulation/xDiscreteElementMethodSimulation.cpp:
63-80): zero velocities, identity Euler parameters, acceleration (0, g_y, 0).
All randomness is seeded.
"""
import os
from dataclasses import dataclass, field

import numpy as np

from . import types as T

G_Y = -9.80665


@dataclass
class Scene:
    np_: int
    ns: int
    pos: np.ndarray            # [np*4]  x, y, z, radius
    vel: np.ndarray            # [ns*3]
    acc: np.ndarray            # [ns*3]
    ep: np.ndarray             # [ns*4]
    ev: np.ndarray             # [ns*4]
    ea: np.ndarray             # [ns*4]
    mass: np.ndarray           # [ns]
    inertia: np.ndarray        # [ns*3]
    dt: float
    cell_size: float
    grid: tuple = (128, 128, 128)
    origin: tuple = (-1.0, -1.0, -1.0)
    gravity: tuple = (0.0, G_Y, 0.0)
    contact_model: int = 1
    pp_cp: T.ContactProperty = None
    planes: list = field(default_factory=list)        # PlaneInfo
    plane_cp: list = field(default_factory=list)      # ContactProperty
    plane_body: list = field(default_factory=list)    # 15-double records
    meshes: list = field(default_factory=list)        # dicts: vlist_local, body, cp
    cylinders: list = field(default_factory=list)     # dicts: cyl (CylinderInfo), body, cp
    cpos: np.ndarray = None    # clusters: [ns*4]
    xci: np.ndarray = None     # clusters: uint32 [nco*4]
    rloc: np.ndarray = None    # clusters: [neach*3]
    name: str = ""
    note: str = ""

    def params(self):
        nco = 0 if self.xci is None else self.xci.size // 4
        return T.make_params(np_=self.np_, dt=self.dt, cell_size=self.cell_size, grid=self.grid,
                             origin=self.origin, gravity=self.gravity,
                             contact_model=self.contact_model,
                             ncluster=self.ns if self.ns != self.np_ else 0, nco=nco,
                             nplane=len(self.planes), ncylinder=len(self.cylinders))

    def copy(self):
        import copy
        return copy.deepcopy(self)


def sphere_mass_inertia(r, rho):
    m = rho * (4.0 / 3.0) * np.pi * r ** 3
    J = (2.0 / 5.0) * m * r ** 2
    return m, np.repeat(J, 3).reshape(-1, 3)


def _init_state(ns, g_y=G_Y):
    vel = np.zeros(ns * 3)
    acc = np.zeros(ns * 3)
    acc[1::3] = g_y
    ep = np.zeros(ns * 4)
    ep[0::4] = 1.0
    return vel, acc, ep, np.zeros(ns * 4), np.zeros(ns * 4)


def default_material(E=1e7, nu=0.3, rest=0.5, fric=0.3, rfric=0.0):
    return T.make_contact_property(E_i=E, E_j=E, nu_i=nu, nu_j=nu, rest=rest, fric=fric, rfric=rfric)


def open_box_planes(x0, x1, y0, y1, z0, z1, first_id=0):
    """Floor and four walls of an open-top box with normals (u1 x u2) pointing
    inside, as the reference's plane contact expects (plane frame of
    xParticlePlaneContact.cpp:96-111)."""
    P = T.plane_from_points
    planes = [
        P(0, (x0, y0, z0), (x0, y0, z1), (x1, y0, z0)),   # floor y = y0, normal +y
        P(1, (x0, y0, z0), (x0, y1, z0), (x0, y0, z1)),   # wall x = x0, normal +x
        P(2, (x1, y0, z0), (x1, y0, z1), (x1, y1, z0)),   # wall x = x1, normal -x
        P(3, (x0, y0, z0), (x1, y0, z0), (x0, y1, z0)),   # wall z = z0, normal +z
        P(4, (x0, y0, z1), (x0, y1, z1), (x1, y0, z1)),   # wall z = z1, normal -z
    ]
    for i, p in enumerate(planes):
        p.id = first_id + i
    return planes


def jittered_lattice(nx, ny, nz, spacing, origin, jitter, rng):
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    # order: x fastest within a layer, then z, then y (layers stacked upward)
    pts = np.stack([ix.transpose(1, 2, 0).ravel(), iy.transpose(1, 2, 0).ravel(),
                    iz.transpose(1, 2, 0).ravel()], axis=1).astype(np.float64)
    pts = np.asarray(origin, float) + pts * spacing
    pts += rng.uniform(-jitter, jitter, size=pts.shape)
    return pts


def sphere_drop(n_per_layer_side=41, layers=6, r=1e-3, rho=2500.0, E=1e7, nu=0.3, rest=0.5, fric=0.3,
                dt=1e-5, box=0.1, seed=1234, spacing_factor=2.4, wall_height=None):
    """10,000-sphere drop of the first configuration: jittered cubic lattice
    (spacing 2.4 r, jitter +-0.1 r), 41 x 41 per layer x 6 layers centred in a
    0.1 x 0.1 m open box of five planes, cell size 2 r."""
    rng = np.random.default_rng(seed)
    sp = spacing_factor * r
    n = n_per_layer_side
    width = (n - 1) * sp
    x0 = -0.5 * width
    pts = jittered_lattice(n, layers, n, sp, (x0, 2.0 * r + 0.5 * sp, x0), 0.1 * r, rng)
    N = pts.shape[0]
    pos = np.zeros((N, 4))
    pos[:, :3] = pts
    pos[:, 3] = r
    m, J = sphere_mass_inertia(np.full(N, r), rho)
    vel, acc, ep, ev, ea = _init_state(N)
    h = wall_height if wall_height is not None else max(0.05, pts[:, 1].max() + 4 * r)
    cp = default_material(E, nu, rest, fric)
    planes = open_box_planes(-0.5 * box, 0.5 * box, 0.0, h, -0.5 * box, 0.5 * box)
    return Scene(np_=N, ns=N, pos=pos.ravel(), vel=vel, acc=acc, ep=ep, ev=ev, ea=ea, mass=m,
                 inertia=J.ravel(), dt=dt, cell_size=2.0 * r, pp_cp=cp, planes=planes,
                 plane_cp=[cp] * len(planes), plane_body=[T.body_record() for _ in planes],
                 name="sphere_drop", note=f"{N} spheres r={r}")


def poly_drop(n, r_min=1e-3, r_max=3e-3, rho=2500.0, E=1e7, nu=0.3, rest=0.5, fric=0.3, dt=1e-5, box=0.1,
              seed=7):
    """Polydisperse drop in the first configuration's open box (0.1 x 0.1 m,
    floor and four walls): n spheres with radii U[r_min, r_max] on a jittered
    cubic lattice of pitch 2.4 r_max (jitter +-0.1 r_max) filling the box's
    footprint layer by layer, walls as tall as the lattice; cell size 2 r_max.
    The member scene of the batched parameter sweep."""
    rng = np.random.default_rng(seed)
    sp = 2.4 * r_max
    side = max(1, int(np.floor((box - 2.0 * r_max) / sp)) + 1)
    layers = int(np.ceil(n / (side * side)))
    width = (side - 1) * sp
    x0 = -0.5 * width
    pts = jittered_lattice(side, layers, side, sp, (x0, 2.0 * r_max + 0.5 * sp, x0), 0.1 * r_max, rng)[:n]
    radii = rng.uniform(r_min, r_max, size=n)
    pos = np.zeros((n, 4))
    pos[:, :3] = pts
    pos[:, 3] = radii
    m, J = sphere_mass_inertia(radii, rho)
    vel, acc, ep, ev, ea = _init_state(n)
    h = max(0.05, pts[:, 1].max() + 4 * r_max)
    cp = default_material(E, nu, rest, fric)
    planes = open_box_planes(-0.5 * box, 0.5 * box, 0.0, h, -0.5 * box, 0.5 * box)
    return Scene(np_=n, ns=n, pos=pos.ravel(), vel=vel, acc=acc, ep=ep, ev=ev, ea=ea, mass=m,
                 inertia=J.ravel(), dt=dt, cell_size=2.0 * r_max, pp_cp=cp, planes=planes,
                 plane_cp=[cp] * len(planes), plane_body=[T.body_record() for _ in planes],
                 name="poly_drop", note=f"{n} spheres r~U[{r_min},{r_max}] fric={fric:.3f} rest={rest:.3f}")


def pow2_at_least(n):
    p = 1
    while p < n:
        p *= 2
    return p


def dam_break(n_target=1_000_000, r_min=1e-3, r_max=2e-3, rho=2500.0, E=1e7, nu=0.3, rest=0.3, fric=0.4,
              dt=5e-6, seed=2024, block_x=0.2, block_z=0.4, box=(1.0, 0.4, 0.4), spacing=None,
              grid="domain"):
    """Polydisperse dam break of the second configuration: radii U[r_min,
    r_max], a block at x in [0, block_x] of a box 1 m long, the gate removed
    at t = 0 (so no gate plane is present).

    The block is a jittered lattice at spacing 2 r_max + 2 jitter + margin so
    no two spheres overlap at t = 0.  Such a lattice holds fewer spheres per
    volume than a settled packing, so the block is as tall as n_target needs
    (about 0.9 m for 1M spheres instead of 0.4 m) and the box walls are raised
    to match; the box keeps its 1 x 0.4 m footprint.

    grid="domain" sizes a non-wrapping power-of-two grid to the box;
    grid="reference" keeps the reference's 128^3 wrapping grid.
    """
    rng = np.random.default_rng(seed)
    jit = 0.02 * r_max
    sp = spacing if spacing is not None else 2.0 * r_max + 2.0 * jit + 0.02 * r_max
    nx = int(np.floor((block_x - 2 * r_max) / sp)) + 1
    nz = int(np.floor((block_z - 2 * r_max) / sp)) + 1
    ny = int(np.ceil(n_target / (nx * nz)))
    # columns on a jittered square pitch sp >= 2 r_max; inside a column each
    # sphere rests on the one below it with an overlap of 1e-3 r_min, so the
    # column carries its weight through contacts from the first step
    radii = rng.uniform(r_min, r_max, size=(ny, nz, nx))
    gap = -1e-3 * r_min
    ys = np.cumsum(radii + np.roll(radii, 1, axis=0) + gap, axis=0) - radii[0:1] - gap
    ys = ys - ys[0:1] + radii[0:1] + gap
    xs = (r_max + jit + np.arange(nx) * sp)[None, None, :] + rng.uniform(-jit, jit, size=(1, nz, nx))
    zs = (r_max + jit + np.arange(nz) * sp)[None, :, None] + rng.uniform(-jit, jit, size=(1, nz, nx))
    pts = np.stack([np.broadcast_to(xs, radii.shape), ys, np.broadcast_to(zs, radii.shape)], axis=-1)
    pts = pts.reshape(-1, 3)[:n_target]
    radii = radii.reshape(-1)[:n_target]
    N = pts.shape[0]
    pos = np.zeros((N, 4))
    pos[:, :3] = pts
    pos[:, 3] = radii
    m, J = sphere_mass_inertia(radii, rho)
    vel, acc, ep, ev, ea = _init_state(N)
    height = max(box[1], pts[:, 1].max() + 2 * r_max)
    cp = default_material(E, nu, rest, fric)
    # floor, walls x = 0 and x = box[0], walls z = 0 and z = box[2]
    planes = open_box_planes(0.0, box[0], 0.0, height + 0.01, 0.0, box[2])
    cs = 2.0 * r_max
    if grid == "domain":
        # origin 1.25 cells below the box; one spare cell above it
        o = -1.25 * cs
        gx = pow2_at_least(int(np.ceil((box[0] - o) / cs)) + 1)
        gy = pow2_at_least(int(np.ceil((height + 0.01 - o) / cs)) + 1)
        gz = pow2_at_least(int(np.ceil((box[2] - o) / cs)) + 1)
        grid_dims = (gx, gy, gz)
        origin = (o, o, o)
    else:
        grid_dims = (128, 128, 128)
        origin = (-1.0, -1.0, -1.0)
    return Scene(np_=N, ns=N, pos=pos.ravel(), vel=vel, acc=acc, ep=ep, ev=ev, ea=ea, mass=m,
                 inertia=J.ravel(), dt=dt, cell_size=cs, grid=grid_dims, origin=origin, pp_cp=cp,
                 planes=planes, plane_cp=[cp] * len(planes),
                 plane_body=[T.body_record() for _ in planes], name="dam_break",
                 note=f"{N} spheres r~U[{r_min},{r_max}] lattice {nx}x{ny}x{nz} spacing {sp:.5g} "
                      f"block height {pts[:, 1].max():.3f} m")


def fcc_block(n, d, x_range, z_range, y0, jitter, rng):
    """n sites of a face-centred cubic lattice with nearest-neighbour
    distance d filling x_range x z_range layer by layer from y0 upward:
    points of the cubic lattice of pitch h = d / sqrt(2) whose index sum is
    even.  Ordered by layer (y), then z, then x, as the reference's cube
    fills number their particles.  Each coordinate is jittered by
    U[-jitter, jitter]."""
    h = d / np.sqrt(2.0)
    nx = int(np.floor((x_range[1] - x_range[0]) / h)) + 1
    nz = int(np.floor((z_range[1] - z_range[0]) / h)) + 1
    per_two = nx * nz  # sites in two consecutive layers
    ny = int(np.ceil(2 * n / per_two)) + 1
    j, k, i = np.meshgrid(np.arange(ny), np.arange(nz), np.arange(nx), indexing="ij")
    keep = ((i + j + k) & 1) == 0
    pts = np.stack([x_range[0] + i[keep] * h, y0 + j[keep] * h, z_range[0] + k[keep] * h], axis=1)[:n]
    if pts.shape[0] < n:
        raise ValueError("fcc_block: lattice too small")
    return pts + rng.uniform(-jitter, jitter, size=pts.shape)


def dam_break_fill(n=1_000_000, r_min=1e-3, r_max=2e-3, rho=2500.0, E=1e7, nu=0.3, rest=0.3, fric=0.4,
                   dt=1e-5, seed=2025, block_x=0.2, box=(1.0, 0.4, 0.4)):
    """The dam-break block before it settles: n spheres with radii
    U[r_min, r_max] (seeded) on a jittered FCC lattice of nearest-neighbour
    distance 2 r_max + 0.1 mm (no two spheres touch) filling x in
    [0, block_x] and the box's depth, in a box of floor, four walls and the
    gate plane at x = block_x, walls as tall as the lattice.  The settling
    pre-run (settle_dam_break) turns it into the random packing the dam
    break starts from."""
    rng = np.random.default_rng(seed)
    d = 2.0 * r_max + 1e-4
    m = r_max + 5e-5
    pts = fcc_block(n, d, (m, block_x - m), (m, box[2] - m), m, 2e-5, rng)
    radii = rng.uniform(r_min, r_max, size=n)
    pos = np.zeros((n, 4))
    pos[:, :3] = pts
    pos[:, 3] = radii
    mass, J = sphere_mass_inertia(radii, rho)
    vel, acc, ep, ev, ea = _init_state(n)
    top = float(pts[:, 1].max()) + 2.0 * r_max
    cp = default_material(E, nu, rest, fric)
    planes = open_box_planes(0.0, box[0], 0.0, top, 0.0, box[2])
    gate = T.plane_from_points(len(planes), (block_x, 0.0, 0.0), (block_x, 0.0, box[2]), (block_x, top, 0.0))
    planes.append(gate)
    cs = 2.0 * r_max
    o = -1.25 * cs
    grid_dims = (pow2_at_least(int(np.ceil((box[0] - o) / cs)) + 1),
                 pow2_at_least(int(np.ceil((top - o) / cs)) + 1),
                 pow2_at_least(int(np.ceil((box[2] - o) / cs)) + 1))
    return Scene(np_=n, ns=n, pos=pos.ravel(), vel=vel, acc=acc, ep=ep, ev=ev, ea=ea, mass=mass,
                 inertia=J.ravel(), dt=dt, cell_size=cs, grid=grid_dims, origin=(o, o, o), pp_cp=cp,
                 planes=planes, plane_cp=[cp] * len(planes), plane_body=[T.body_record() for _ in planes],
                 name="dam_break_fill", note=f"{n} spheres r~U[{r_min},{r_max}] FCC fill, top {top:.3f} m")


# Settling pre-run of the dam-break packing: block shapes of the mixed step
# (they do not change results) and the number of settling steps of 1e-5 s.
SETTLE_SHAPES = dict(nt_pairs=128, stage=8, nt_bodies=128, occ_pairs=1024, occ_bodies=768, skin_div=32)
SETTLE_STEPS = 40000


def cache_dir():
    d = os.environ.get("XDEM_CACHE") or os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                                     ".xdem_cache")
    os.makedirs(d, exist_ok=True)
    return d


def settle_dam_break(fill, steps, path, log=None):
    """Untimed, seeded settling pre-run on the GPU: the FCC fill falls under
    gravity behind the gate and comes to rest as a random packing (mixed
    step, dt of the fill).  Writes the final state and the particle-pair and
    plane pair lists with their tangential history to a part file (the
    reference's version-2 layout) at `path`.  Deterministic: the step sums
    every contact in a fixed order, so the same build on the same GPU model
    writes the same file."""
    from . import sim as S
    sm = S.Sim(fill, precision=T.XDEM_MIXED)
    sm.set_tune(**SETTLE_SHAPES)
    sm.set_graph(True)
    done = 0
    chunk = 5000
    while done < steps:
        k = min(chunk, steps - done)
        sm.step(k)
        done += k
        if log:
            ke, nc = sm.energy()
            log(f"settle {done}/{steps}: ke {ke:.4e} J, {nc / fill.np_:.3f} contacts/sphere, "
                f"status {sm.status()}")
    tmp = path + ".tmp"
    sm.save_part(tmp, 0.0)
    sm.close()
    os.replace(tmp, path)


def dam_break_packed(n=1_000_000, seed=2025, settle_steps=SETTLE_STEPS, dt=5e-6, box=(1.0, 0.4, 0.4),
                     log=None, path=None):
    """The dam-break configuration from a settled random packing: the FCC
    fill of dam_break_fill settled behind the gate for `settle_steps` steps
    of 1e-5 s (settle_dam_break, cached as a part file keyed by n, seed and
    steps), then the gate removed (t = 0).  The box is 1 x 0.4 x 0.4 m
    (floor, four walls 0.4 m tall); dt 5e-6 s.  The scene carries the
    settled state and, in `pairs`, the particle-pair and plane lists with
    their tangential history (kinds 0 and 1; the gate's slots are dropped
    by the first step, whose plane 0 restarts every plane list)."""
    from . import partfile
    fill = dam_break_fill(n=n, seed=seed, box=box)
    if path is None:
        path = os.path.join(cache_dir(), f"dam_break_n{n}_s{seed}_k{settle_steps}.part")
    if not os.path.exists(path):
        settle_dam_break(fill, settle_steps, path, log=log)
    d = partfile.read(path, ("pp", "pl"))
    if d["np"] != n:
        raise ValueError(f"{path}: {d['np']} spheres, {n} expected")
    sc = fill.copy()
    sc.pos, sc.vel, sc.acc = d["pos"], d["vel"], d["acc"]
    sc.ep, sc.ev, sc.ea = d["ep"], d["ev"], d["ea"]
    sc.dt = dt
    sc.planes = open_box_planes(0.0, box[0], 0.0, box[1], 0.0, box[2])
    sc.plane_cp = [sc.pp_cp] * len(sc.planes)
    sc.plane_body = [T.body_record() for _ in sc.planes]
    cap_pp, cap_pl = T.MAX_P2P_COUNT, T.MAX_P2PL_COUNT
    # the gate is gone: its plane slots are dropped, the other planes' slots
    # keep their order and history
    nb = len(sc.planes)
    plc, pli, plt = d["pl_count"], d["pl_id"].reshape(n, cap_pl), d["pl_tsd"].reshape(n, cap_pl, 2)
    keep = (np.arange(cap_pl)[None, :] < plc[:, None]) & (pli < nb)
    order = np.argsort(~keep, axis=1, kind="stable")
    pli = np.where(np.take_along_axis(keep, order, 1), np.take_along_axis(pli, order, 1), 0)
    plt = np.where(np.take_along_axis(keep, order, 1)[:, :, None], np.take_along_axis(plt, order[:, :, None], 1), 0.0)
    plc = keep.sum(1).astype(np.uint32)
    sc.pairs = [(d["pp_count"], d["pp_id"], d["pp_tsd"]), (plc, pli.ravel(), plt.ravel())]
    assert d["pp_id"].size == n * cap_pp and d["pl_id"].size == n * cap_pl
    p = sc.pos.reshape(-1, 4)
    sc.name = "dam_break_packed"
    sc.note = (f"{n} spheres r~U[1,2] mm, random packing settled {settle_steps} x 1e-5 s behind the gate "
               f"(bed top {float((p[:, 1] + p[:, 3]).max()):.3f} m), gate removed at t = 0")
    sc.part_path = path
    return sc


def random_packed(n, r_min, r_max, box, seed, overlap=0.05, vel_scale=0.05, omega_scale=5.0,
                  cell_factor=2.0, grid=(128, 128, 128), origin=(-1.0, -1.0, -1.0), rho=2500.0,
                  E=1e7, nu=0.3, rest=0.5, fric=0.3, dt=1e-5, rfric=0.0, nplanes=5):
    """Dense random spheres with overlaps, random velocities and spins: a
    single-step test bed where most spheres have several contacts.  The
    lattice spacing is chosen so neighbours overlap by up to `overlap` of
    the radius."""
    rng = np.random.default_rng(seed)
    sp = 2.0 * r_max * (1.0 - overlap)
    side = int(np.ceil(n ** (1.0 / 3.0)))
    pts = jittered_lattice(side, side, side, sp, (-0.5 * side * sp, r_max, -0.5 * side * sp),
                           0.15 * r_max, rng)[:n]
    radii = rng.uniform(r_min, r_max, size=n)
    pos = np.zeros((n, 4))
    pos[:, :3] = pts
    pos[:, 3] = radii
    m, J = sphere_mass_inertia(radii, rho)
    vel = rng.normal(0, vel_scale, size=(n, 3)).ravel()
    acc = np.zeros(n * 3)
    acc[1::3] = G_Y
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w = rng.normal(0, omega_scale, size=(n, 3))
    # e_dot = 1/2 G(e)^T omega with G rows of the angular-velocity map (impl:32-41)
    e0, e1, e2, e3 = q.T
    G = np.stack([np.stack([-e1, e0, -e3, e2], 1), np.stack([-e2, e3, e0, -e1], 1),
                  np.stack([-e3, -e2, e1, e0], 1)], 1)  # [n,3,4]
    ed = 0.5 * np.einsum("nij,ni->nj", G, w)
    ea = rng.normal(0, 1.0, size=(n, 4)) * 1e-3
    cp = default_material(E, nu, rest, fric, rfric)
    lo = pts.min(0) - r_max
    hi = pts.max(0) + r_max
    # planes cut through the outer layer so boundary spheres touch them
    planes = open_box_planes(lo[0] + 0.6 * r_max, hi[0] - 0.6 * r_max, lo[1] + 0.6 * r_max, hi[1] + 0.05,
                             lo[2] + 0.6 * r_max, hi[2] - 0.6 * r_max)[:nplanes]
    return Scene(np_=n, ns=n, pos=pos.ravel(), vel=vel, acc=acc, ep=q.ravel(), ev=ed.ravel(),
                 ea=ea.ravel(), mass=m, inertia=J.ravel(), dt=dt, cell_size=cell_factor * r_max,
                 grid=grid, origin=origin, pp_cp=cp, planes=planes, plane_cp=[cp] * len(planes),
                 plane_body=[T.body_record() for _ in planes], name="random_packed")


def cluster_mass_inertia(rloc, sub_r, rho):
    """Mass and principal inertia of a clump of equal spheres at body-frame
    offsets rloc [neach, 3], as xParticleManager::SetClusterMassAndInertia
    (source/xdynamics_manager/xParticleManager.cpp:1071-1084) sets them:
    m = neach rho 4/3 pi r^3 and J = sum over members of m_s (parallel-axis
    terms of rloc) -- the members' own 2/5 m_s r^2 is computed there but not
    added.  On an axis where that sum is zero (members in a row along it,
    the clumps of the wheel testbed) the reference's value would leave the
    Euler-parameter update dividing by zero; there, and only there, the
    members' own 2/5 m_s r^2 is added.  Returns (mass, J3, axes that got the
    members' own term)."""
    rloc = np.asarray(rloc, float).reshape(-1, 3)
    neach = rloc.shape[0]
    m1 = rho * (4.0 / 3.0) * np.pi * sub_r ** 3
    J3 = np.array([m1 * np.sum(rloc[:, 1] ** 2 + rloc[:, 2] ** 2), m1 * np.sum(rloc[:, 0] ** 2 + rloc[:, 2] ** 2),
                   m1 * np.sum(rloc[:, 0] ** 2 + rloc[:, 1] ** 2)])
    own = J3 == 0.0
    J3 = np.where(own, (2.0 / 5.0) * m1 * sub_r ** 2 * neach, J3)
    return m1 * neach, J3, own


def cluster_bed(ncluster, neach=3, sub_r=2e-3, seed=7, rho=2500.0, E=1e7, nu=0.3, rest=0.5, fric=0.3,
                dt=1e-5, spacing_factor=1.0, trough=(1.0, 0.3, 0.15), vel_scale=0.0, grid=(128, 128, 128),
                origin=(-1.0, -1.0, -1.0), cell_size=None):
    """Bed of rigid multi-sphere clumps (neach spheres in a row, touching,
    seeded random orientation) on a jittered lattice in a trough of five
    planes; cluster table, member offsets and mass/inertia as
    xParticleManager::SetClusterMassAndInertia (xParticleManager.cpp:
    1058-1101)."""
    rng = np.random.default_rng(seed)
    rloc = np.zeros((neach, 3))
    rloc[:, 0] = (np.arange(neach) - 0.5 * (neach - 1)) * 2.0 * sub_r * 0.95
    reach = float(np.abs(rloc[:, 0]).max()) + sub_r
    sp = 2.0 * reach * spacing_factor + 0.1 * sub_r
    nx = max(1, int(np.floor((trough[0] - 2 * reach) / sp)) + 1)
    nz = max(1, int(np.floor((trough[2] - 2 * reach) / sp)) + 1)
    ny = int(np.ceil(ncluster / (nx * nz)))
    cent = jittered_lattice(nx, ny, nz, sp, (reach, reach, reach), 0.02 * sub_r, rng)[:ncluster]
    ns = cent.shape[0]
    q = rng.normal(size=(ns, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    cpos = np.zeros((ns, 4))
    cpos[:, :3] = cent
    cpos[:, 3] = sub_r
    # member positions = c + A(q) rloc
    e0, e1, e2, e3 = q.T
    A = np.empty((ns, 3, 3))
    A[:, 0] = np.stack([2 * (e0 * e0 + e1 * e1 - 0.5), 2 * (e1 * e2 - e0 * e3), 2 * (e1 * e3 + e0 * e2)], 1)
    A[:, 1] = np.stack([2 * (e1 * e2 + e0 * e3), 2 * (e0 * e0 + e2 * e2 - 0.5), 2 * (e2 * e3 - e0 * e1)], 1)
    A[:, 2] = np.stack([2 * (e1 * e3 - e0 * e2), 2 * (e2 * e3 + e0 * e1), 2 * (e0 * e0 + e3 * e3 - 0.5)], 1)
    mem = cent[:, None, :] + np.einsum("nij,kj->nki", A, rloc)
    N = ns * neach
    pos = np.zeros((N, 4))
    pos[:, :3] = mem.reshape(-1, 3)
    pos[:, 3] = sub_r
    m_c, J3, _ = cluster_mass_inertia(rloc, sub_r, rho)
    mass = np.full(ns, m_c)
    inertia = np.tile(J3, ns)
    vel, acc, ep, ev, ea = _init_state(ns)
    ep = q.ravel().copy()
    if vel_scale:
        vel = rng.normal(0, vel_scale, size=ns * 3)
    xci = np.array([0, 0, ns, neach], dtype=np.uint32)
    height = max(trough[1], cent[:, 1].max() + 2 * reach)
    cp = default_material(E, nu, rest, fric)
    planes = open_box_planes(0.0, trough[0], 0.0, height + 0.01, 0.0, trough[2])
    return Scene(np_=N, ns=ns, pos=pos.ravel(), vel=vel, acc=acc, ep=ep, ev=ev, ea=ea, mass=mass,
                 inertia=inertia, dt=dt, cell_size=cell_size or 2.0 * sub_r, grid=grid, origin=origin,
                 pp_cp=cp, planes=planes, plane_cp=[cp] * len(planes),
                 plane_body=[T.body_record() for _ in planes], cpos=cpos.ravel(), xci=xci,
                 rloc=rloc.ravel(), name="cluster_bed", note=f"{ns} clusters x {neach}")


def uv_sphere_mesh(radius, n_lat, n_lon):
    """Closed triangle mesh of a sphere (body frame), vertices P,Q,R per
    triangle as the vertex list xParticleMeshObjectContact::define uploads."""
    tris = []
    for i in range(n_lat):
        t0 = np.pi * i / n_lat
        t1 = np.pi * (i + 1) / n_lat
        for j in range(n_lon):
            p0 = 2 * np.pi * j / n_lon
            p1 = 2 * np.pi * (j + 1) / n_lon

            def v(t, p):
                return radius * np.array([np.sin(t) * np.cos(p), np.cos(t), np.sin(t) * np.sin(p)])
            a, b, c, d = v(t0, p0), v(t1, p0), v(t1, p1), v(t0, p1)
            if i > 0:
                tris.append((a, b, d))
            if i < n_lat - 1:
                tris.append((b, c, d))
    return np.array(tris, dtype=np.float64).reshape(-1, 9)


def wheel_mesh(radius=0.15, width=0.1, n_around=100, n_width=4):
    """Closed cylinder (wheel) mesh in its body frame, axis along z: side
    surface plus two capped discs."""
    tris = []
    zs = np.linspace(-0.5 * width, 0.5 * width, n_width + 1)
    ang = 2 * np.pi * np.arange(n_around + 1) / n_around
    ring = np.stack([radius * np.cos(ang), radius * np.sin(ang)], 1)
    for k in range(n_width):
        for j in range(n_around):
            a = (*ring[j], zs[k]); b = (*ring[j + 1], zs[k])
            c = (*ring[j + 1], zs[k + 1]); d = (*ring[j], zs[k + 1])
            tris.append((a, b, c))
            tris.append((a, c, d))
    for z, sgn in ((zs[0], -1), (zs[-1], 1)):
        for j in range(n_around):
            o = (0.0, 0.0, z)
            a = (*ring[j], z); b = (*ring[j + 1], z)
            tris.append((o, b, a) if sgn < 0 else (o, a, b))
    return np.array(tris, dtype=np.float64).reshape(-1, 9)


def tyre_mesh(radius=0.15, width=0.1, n_around=320, n_width=32):
    """Tyre surface of a wheel (open cylinder, axis along z, body frame):
    n_around x n_width quads, each split into two triangles, wound so that
    the normals (P->Q x P->R) point outward."""
    ang = 2 * np.pi * np.arange(n_around + 1) / n_around
    zs = np.linspace(-0.5 * width, 0.5 * width, n_width + 1)
    cx, cy = radius * np.cos(ang), radius * np.sin(ang)
    tris = np.empty((n_around * n_width * 2, 9))
    t = 0
    for k in range(n_width):
        for j in range(n_around):
            a = (cx[j], cy[j], zs[k]); b = (cx[j + 1], cy[j + 1], zs[k])
            c = (cx[j + 1], cy[j + 1], zs[k + 1]); d = (cx[j], cy[j], zs[k + 1])
            tris[t] = (*a, *c, *b)
            tris[t + 1] = (*a, *d, *c)
            t += 2
    return tris


def fit_sphere_radius(tris, ft=0.8):
    """Radius of the sphere FitSphereToTriangle(P, Q, R, ft) fits to each
    triangle (xUtilityFunction.cpp:379-416): its iteration converges to the
    sphere through the circumcircle whose centre lies on the normal at
    distance d with d / r = ft, i.e. r = (circumradius) / sqrt(1 - ft^2)."""
    P, Q, R = tris[:, 0:3], tris[:, 3:6], tris[:, 6:9]
    a = np.linalg.norm(Q - R, axis=1)
    b = np.linalg.norm(R - P, axis=1)
    c = np.linalg.norm(P - Q, axis=1)
    area = 0.5 * np.linalg.norm(np.cross(Q - P, R - P), axis=1)
    return (a * b * c) / (4.0 * area) / np.sqrt(1.0 - ft * ft)


def wheel_testbed(ncluster=2_000_000, neach=3, sub_r=2e-3, rho=2500.0, E=1e7, nu=0.3, rest=0.5, fric=0.3,
                  dt=1e-5, trough=(1.0, 0.3, 0.15), wheel_r=0.15, wheel_w=0.1, n_around=320, n_width=32,
                  omega=2.0, wheel_mass=20.0, sink=1e-4, seed=2024):
    """Wheel on a bed of rigid clumps of `neach` spheres (sub-radius sub_r)
    in a trough of five planes, x along the trough.

    Clumps lie along x (members 1.9 sub_r apart, as cluster_bed) with a
    seeded spin about that axis, in columns: clumps of one column touch with
    1e-3 sub_r overlap (so every member has a contact above and below from
    t = 0), neighbouring columns are 0.1 mm apart in z and 0.2 mm end to end
    in x.  Clumps are numbered layer by layer, x fastest, so that clumps
    touching in a column are far apart in id and the reference's skip of
    partners with |id - k| <= neach (impl:556-558) drops none of their
    contacts.  The bed fills the trough's footprint and rises above it: the
    walls are extended to the bed's height (2,000,000 clumps of 2 mm spheres
    stand about 2.6 m tall on a 1.0 x 0.15 m floor).

    The wheel: a tyre surface of n_around x n_width quads (20,480 triangles
    by default) of radius wheel_r and width wheel_w, axis along z, centred
    over the trough at x = trough/2, sunk `sink` (0.1 mm: the spheres of
    the top layer within about 5 mm of the tyre's lowest line touch it) into
    the top of the bed's last complete layer, driven at `omega` rad/s
    (rolling toward +x) through its body record.  Its
    surface is invariant under rotation about the axis, so the drive needs
    no re-posing of the triangles between steps.  The cell size follows
    xDiscreteElementMethodSimulation.cpp:91-99: twice the largest radius of
    particles and mesh spheres."""
    rng = np.random.default_rng(seed)
    sp = 2.0 * sub_r * 0.95
    rloc = np.zeros((neach, 3))
    rloc[:, 0] = (np.arange(neach) - 0.5 * (neach - 1)) * sp
    half = float(np.abs(rloc[:, 0]).max()) + sub_r
    px = 2.0 * half + 2e-4
    pz = 2.0 * sub_r + 1e-4
    py = 2.0 * sub_r * (1.0 - 1e-3)
    nx = max(1, int(np.floor(trough[0] / px)))
    nz = max(1, int(np.floor(trough[2] / pz)))
    per_layer = nx * nz
    ny = -(-ncluster // per_layer)
    k = np.arange(ncluster)
    ix, iz, iy = k % nx, (k // nx) % nz, k // per_layer
    x0 = 0.5 * (trough[0] - nx * px)
    z0 = 0.5 * (trough[2] - nz * pz)
    cent = np.stack([x0 + (ix + 0.5) * px, sub_r * (1.0 - 1e-3) + iy * py, z0 + (iz + 0.5) * pz], 1)
    # spin about x: e = (cos a/2, sin a/2, 0, 0)
    a = rng.uniform(0.0, 2.0 * np.pi, ncluster)
    q = np.zeros((ncluster, 4))
    q[:, 0] = np.cos(0.5 * a)
    q[:, 1] = np.sin(0.5 * a)
    ns = ncluster
    N = ns * neach
    pos = np.empty((N, 4))
    pos[:, 0] = (cent[:, None, 0] + rloc[None, :, 0]).ravel()
    pos[:, 1] = np.repeat(cent[:, 1], neach)
    pos[:, 2] = np.repeat(cent[:, 2], neach)
    pos[:, 3] = sub_r
    cpos = np.zeros((ns, 4))
    cpos[:, :3] = cent
    cpos[:, 3] = sub_r
    m_c, J3, _ = cluster_mass_inertia(rloc, sub_r, rho)
    mass = np.full(ns, m_c)
    inertia = np.tile(J3, ns)
    vel, acc, ep, ev, ea = _init_state(ns)
    ep = q.ravel().copy()
    xci = np.array([0, 0, ns, neach], dtype=np.uint32)
    # the wheel rests on the last complete layer (a partial top layer fills
    # rows from z = 0 and need not reach under the tyre)
    full = max(1, ncluster // per_layer)
    top = sub_r * (1.0 - 1e-3) + (full - 1) * py + sub_r
    tyre = tyre_mesh(wheel_r, wheel_w, n_around, n_width)
    r_ms = float(fit_sphere_radius(tyre).max())
    cell = 2.0 * max(sub_r, r_ms)
    wc = (0.5 * trough[0], top + wheel_r - sink, 0.5 * trough[2])
    height = max(trough[1], wc[1] + wheel_r + 0.05)
    cp = default_material(E, nu, rest, fric)
    planes = open_box_planes(0.0, trough[0], 0.0, height, 0.0, trough[2])
    origin = (-0.02, -0.02, -0.02)
    grid = tuple(pow2_at_least(int(np.ceil((ext + 0.04) / cell)) + 1) for ext in (trough[0], height, trough[2]))
    body = T.body_record(mass=wheel_mass, pos=wc, ed=(0.0, 0.0, 0.0, -0.5 * omega))
    return Scene(np_=N, ns=ns, pos=pos.ravel(), vel=vel, acc=acc, ep=ep, ev=ev, ea=ea, mass=mass,
                 inertia=inertia, dt=dt, cell_size=cell, grid=grid, origin=origin, pp_cp=cp, planes=planes,
                 plane_cp=[cp] * len(planes), plane_body=[T.body_record() for _ in planes],
                 meshes=[dict(vlist_local=tyre, body=body, cp=cp)], cpos=cpos.ravel(), xci=xci,
                 rloc=rloc.ravel(), name="wheel_testbed",
                 note=f"{ns} clumps x {neach} spheres, {ny} layers, tyre {tyre.shape[0]} triangles")


def column_collapse(n_target=65536, r=1.5e-3, R=0.1, H=0.3, rho=2500.0, E=1e7, nu=0.3, rest=0.5, fric=0.3,
                    dt=1e-5, seed=5150, v0=0.0, floor_half=0.5, jitter=0.1):
    """Column collapse of the differentiable-calibration configuration:
    about n_target spheres of radius r on a seeded jittered cubic lattice
    (jitter +-jitter r) filling a vertical cylinder of radius R and height H
    that stands on a floor plane (a 2 floor_half square at y = 0, normal +y);
    no cylinder wall, so the column collapses once released.  The lattice
    spacing is the largest (never below 2.2 r) that puts at least n_target
    sites inside the cylinder; v0 is an optional initial downward speed."""
    rng = np.random.default_rng(seed)

    def layout(sp):
        nxz = int(np.floor(2.0 * R / sp)) + 1
        ny = max(1, int(np.floor((H - 2.0 * r) / sp)) + 1)
        x0 = -0.5 * (nxz - 1) * sp
        c = x0 + sp * np.arange(nxz)
        inside = int(((c[:, None] ** 2 + c[None, :] ** 2) <= (R - r) ** 2).sum())
        return nxz, ny, x0, inside * ny

    sp = max(2.2 * r, (np.pi * R * R * H / n_target) ** (1.0 / 3.0))
    while sp > 2.2 * r and layout(sp)[3] < n_target:
        sp = max(2.2 * r, sp * 0.995)
    nxz, ny, x0, _ = layout(sp)
    pts = jittered_lattice(nxz, ny, nxz, sp, (x0, r + 0.5 * sp, x0), jitter * r, rng)
    keep = pts[:, 0] ** 2 + pts[:, 2] ** 2 <= (R - r) ** 2
    pts = pts[keep]
    N = pts.shape[0]
    pos = np.zeros((N, 4))
    pos[:, :3] = pts
    pos[:, 3] = r
    m, J = sphere_mass_inertia(np.full(N, r), rho)
    vel, acc, ep, ev, ea = _init_state(N)
    vel[1::3] = -abs(v0)
    cp = default_material(E, nu, rest, fric)
    f = floor_half
    planes = [T.plane_from_points(0, (-f, 0.0, -f), (-f, 0.0, f), (f, 0.0, -f))]
    cs = 2.0 * r
    extent = max(2.0 * (R + 0.05), H + 0.02)
    g = pow2_at_least(int(np.ceil(extent / cs)))
    grid = (g, g, g)
    origin = (-0.5 * g * cs, -2.0 * cs, -0.5 * g * cs)
    return Scene(np_=N, ns=N, pos=pos.ravel(), vel=vel, acc=acc, ep=ep, ev=ev, ea=ea, mass=m,
                 inertia=J.ravel(), dt=dt, cell_size=cs, grid=grid, origin=origin, pp_cp=cp, planes=planes,
                 plane_cp=[cp], plane_body=[T.body_record()], name="column_collapse",
                 note=f"{N} spheres r={r} in a cylinder R={R} H={H}")
