"""Synthetic aggregate setups in PeriDEM's setup schema.

Particles are jittered cubic lattices clipped to a shape, with nodal volume h^3. Bonds follow
exp_dict.py:544-567: every node pair with distance <= delta, as
sorted(cKDTree(pos).query_pairs(delta)). Material constants use the 3D Silling-Askari
formulas of material_dict.py:266-277 (cnot = 18K/(pi delta^4), snot = sqrt(5 G0/(9 K delta)),
K = E/(3(1-2 nu))). The contact stiffness follows the examples' rule
normal_stiffness = peridem_3d(contact_radius).cnot / contact_radius
(examples/3D-HPC-aggregate-particle-breakage/setup.py:160), lowered when it would make the
explicit contact update unstable at the configured dt; the value used is stored in the setup.

Named workloads (seeded):
  two_sphere   two R = 1 mm glass spheres, h = 0.1 mm, B moving at 20 m/s, dt 1e-8, 2000 steps
  cubes125     5x5x5 randomly rotated 1 mm glass cubes, h = 0.125 mm, box walls, gravity
               x1e4, dt 2e-8, 20000 steps
  crush512     512 spheres/cubes/ellipsoids, sizes U[0.6, 1.4] mm, h from {0.05, 0.075, 0.1}
               mm, 12 mm box whose top wall moves down at 1 m/s, dt 5e-9, 10000 steps
  notched_plate  100 x 200 x 9 mm steel plate with two 50 mm x 1.5 mm edge notches, h = 0.5 mm,
               hit between the notches by a 50 mm wide steel block at 32 m/s, dt 2e-8, 5000 steps
  crush_contact  crush512_4m's first 16 particles on a 1.2 mm pitch, touching, pressed by the top
               wall at 20 m/s: contact and breaking from the first steps (accuracy under fracture)
"""
from __future__ import annotations

import math

import numpy as np

from .setupdata import Setup, concat

GLASS = dict(E=72e9, nu=0.25, rho=2440.0, G0=135.0)
STEEL = dict(E=190e9, nu=0.3, rho=8000.0, G0=22170.0)
MM = 1e-3


def material_3d(mat: dict, delta: float) -> dict:
    K = mat["E"] / (3 * (1 - 2 * mat["nu"]))
    return dict(rho=mat["rho"], delta=delta, cnot=18 * K / (np.pi * delta ** 4),
                snot=float(np.sqrt(5 * mat["G0"] / (9 * K * delta))))


def kn_rule(Rc: float) -> float:
    """peridem_3d(Rc).cnot / Rc with the bulk modulus 2e9 of material_dict.peridem_3d."""
    return (18 * 2.0e9 / (np.pi * Rc ** 4)) / Rc


def stable_kn(Kn: float, rho_min: float, vol_max: float, dt: float, frac: float = 0.1) -> float:
    return float(min(Kn, frac * rho_min / (vol_max * dt * dt)))


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def lattice(kind: str, size, h: float) -> np.ndarray:
    """Cubic lattice points of spacing h inside a shape centred at the origin.
    kind: 'sphere' (size = diameter), 'cube' (edge), 'ellipsoid' (3 diameters),
    'box' (3 edges)."""
    if kind in ("cube", "box"):
        e = np.broadcast_to(np.asarray(size, dtype=np.float64), (3,))
        ax = [(np.arange(max(1, int(round(ek / h)))) + 0.5) * h - ek / 2 for ek in e]
        X, Y, Z = np.meshgrid(*ax, indexing="ij")
        return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    d = np.broadcast_to(np.asarray(size, dtype=np.float64), (3,))
    r = d / 2
    n = [int(math.ceil(rk / h)) for rk in r]
    ax = [np.arange(-nk, nk + 1) * h for nk in n]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    P = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    keep = ((P / r) ** 2).sum(axis=1) <= 1.0 + 1e-12
    return P[keep]


_BOND_BUILDER = "cpu"


def set_bond_builder(kind: str):
    """'cpu': scipy cKDTree (the reference's own call); 'gpu': pd_query_pairs on the current
    CUDA device (the same pairs, tested equal)."""
    global _BOND_BUILDER
    if kind not in ("cpu", "gpu"):
        raise ValueError(kind)
    _BOND_BUILDER = kind


def bonds_gpu(positions: list, radii: list) -> list:
    """Pair lists of several point sets in one GPU call (pd_query_pairs): for each set, the
    sorted (i, j), i < j, with |x_i - x_j| <= r."""
    import ctypes as C
    from ._capi import lib, ptr
    L = lib()
    P = len(positions)
    off = np.zeros(P + 1, dtype=np.uint64)
    off[1:] = np.cumsum([len(x) for x in positions])
    pos = np.ascontiguousarray(np.concatenate([np.asarray(x, dtype=np.float64).reshape(-1, 3) for x in positions])
                               if P else np.zeros((0, 3)))
    rad = np.ascontiguousarray(radii, dtype=np.float64)
    po = np.zeros(P + 1, dtype=np.uint64)
    rc = L.pd_query_pairs(ptr(pos), ptr(off), ptr(rad), P, None, 0, ptr(po))
    if rc != 0:
        raise RuntimeError(f"pd_query_pairs: [{rc}] {L.pd_pairs_error().decode()}")
    M = int(po[-1])
    out = np.zeros((max(M, 1), 2), dtype=np.uint32)
    rc = L.pd_query_pairs(ptr(pos), ptr(off), ptr(rad), P, ptr(out), M, ptr(po))
    if rc != 0:
        raise RuntimeError(f"pd_query_pairs: [{rc}] {L.pd_pairs_error().decode()}")
    return [out[int(po[p]):int(po[p + 1])].copy() for p in range(P)]


def bonds(pos: np.ndarray, delta: float) -> np.ndarray:
    """sorted(cKDTree(pos).query_pairs(delta)) as an (M,2) array (exp_dict.py:544-567)."""
    if _BOND_BUILDER == "gpu":
        return bonds_gpu([pos], [delta])[0]
    from scipy.spatial import cKDTree
    pr = cKDTree(pos).query_pairs(delta, output_type="ndarray")
    if len(pr) == 0:
        return np.zeros((0, 2), dtype=np.uint32)
    order = np.lexsort((pr[:, 1], pr[:, 0]))
    return pr[order].astype(np.uint32)


def boundary_nodes(pos: np.ndarray, conn: np.ndarray, Rc: float) -> np.ndarray:
    """Nodes within Rc of a surface node (gen_nonlocal_boundry_nodes, exp_dict.py:1231-1248),
    ascending; surface nodes are those with a degree below 90% of the particle's maximum. The
    test is the reference's, sqrt((dx*dx + dy*dy) + dz*dz) <= Rc in FP64: candidates from a k-d
    tree (CPU builder) or pd_query_near (GPU builder), the same set."""
    n = len(pos)
    deg = np.bincount(conn.reshape(-1).astype(np.int64), minlength=n) if len(conn) else np.zeros(n, int)
    marked = deg < 0.9 * max(1, deg.max())
    if not marked.any():
        return np.zeros(0, np.uint32)
    if _BOND_BUILDER == "gpu":
        return np.nonzero(near_gpu([pos], [marked], [Rc])[0])[0].astype(np.uint32)
    from scipy.spatial import cKDTree
    edge = np.nonzero(marked)[0]
    hits = cKDTree(pos).query_ball_point(pos[edge], Rc * (1.0 + 1e-9))
    near = np.zeros(n, dtype=bool)
    for e, lst in zip(edge, hits):
        if not lst:
            continue
        j = np.asarray(lst, dtype=np.int64)
        d = pos[j] - pos[e]
        near[j[np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]) <= Rc]] = True
    return np.nonzero(near)[0].astype(np.uint32)


def near_gpu(positions: list, marked: list, radii: list) -> list:
    """For each point set, a bool per point: within r of one of the set's marked points
    (pd_query_near, one GPU call for all sets)."""
    from ._capi import lib, ptr
    L = lib()
    P = len(positions)
    off = np.zeros(P + 1, dtype=np.uint64)
    off[1:] = np.cumsum([len(x) for x in positions])
    pos = np.ascontiguousarray(np.concatenate([np.asarray(x, dtype=np.float64).reshape(-1, 3) for x in positions])
                               if P else np.zeros((0, 3)))
    mk = np.ascontiguousarray(np.concatenate([np.asarray(m, dtype=np.uint8) for m in marked]) if P
                              else np.zeros(0, np.uint8))
    rad = np.ascontiguousarray(radii, dtype=np.float64)
    out = np.zeros(max(int(off[-1]), 1), dtype=np.uint8)
    rc = L.pd_query_near(ptr(pos), ptr(off), ptr(rad), P, ptr(mk), ptr(out))
    if rc != 0:
        raise RuntimeError(f"pd_query_near: [{rc}] {L.pd_pairs_error().decode()}")
    return [out[int(off[p]):int(off[p + 1])].astype(bool) for p in range(P)]


def make_particle(local: np.ndarray, h: float, mat: dict, delta_factor: float, rng, jitter: float,
                  center, rotation=None, vel=(0, 0, 0), Rc: float | None = None, **flags) -> dict:
    P = local.copy()
    if rotation is not None:
        P = P @ rotation.T
    if jitter:
        P = P + rng.uniform(-jitter * h, jitter * h, size=P.shape)
    P = P + np.asarray(center, dtype=np.float64)
    delta = delta_factor * h
    m = material_3d(mat, delta)
    # without a boundary-node pass nothing here needs the bonds yet: finish() builds the
    # pending ones of all particles at once (on all host cores with the CPU builder)
    conn = bonds(P, delta) if Rc is not None else _PendingBonds(P, delta)
    n = len(P)
    part = dict(pos=P, vol=np.full(n, h ** 3), conn=conn, vel=np.tile(np.asarray(vel, float), (n, 1)), **m)
    part["h"] = h
    if Rc is not None:
        part["bdry"] = boundary_nodes(P, conn, Rc)
    part.update(flags)
    return part


class _PendingBonds:
    """Bonds of one particle, built later by resolve_bonds."""

    def __init__(self, pos: np.ndarray, delta: float):
        self.pos, self.delta = pos, delta


def resolve_bonds(parts: list) -> None:
    """Builds every pending bond list of `parts` in place. The CPU builder runs the particles on
    a thread pool (cKDTree releases the GIL while it queries); the GPU builder takes all of
    them in one pd_query_pairs call. The pairs are those bonds() gives one particle at a time."""
    idx = [i for i, p in enumerate(parts) if isinstance(p.get("conn"), _PendingBonds)]
    if not idx:
        return
    jobs = [parts[i]["conn"] for i in idx]
    if _BOND_BUILDER == "gpu":
        out = bonds_gpu([j.pos for j in jobs], [j.delta for j in jobs])
    else:
        import os
        from concurrent.futures import ThreadPoolExecutor
        with ThreadPoolExecutor(max_workers=max(1, min(32, os.cpu_count() or 1))) as ex:
            out = list(ex.map(lambda j: bonds(j.pos, j.delta), jobs))
    for i, c in zip(idx, out):
        parts[i]["conn"] = c


def finish(parts, Rc, dt, zeta=0.8, mu=0.3, wall=None, kn=None) -> Setup:
    resolve_bonds(parts)
    vol_max = max(float(np.max(p["vol"])) for p in parts)
    rho_min = min(p["rho"] for p in parts)
    Kn = kn if kn is not None else stable_kn(kn_rule(Rc), rho_min, vol_max, dt)
    if wall is None:
        # walls off, but with a geometry: load_wall<3> leaves the wall fields unset when
        # geom_wall_info has a single entry (load_hdf5.h:159-177)
        wall = dict(allow=0, geom=[-1.0, -1.0, -1.0, 1.0, 1.0, 1.0])
    s = concat(parts, dict(contact_radius=Rc, normal_stiffness=Kn, damping_ratio=zeta,
                           friction_coefficient=mu), wall)
    s.meta["h"] = [p["h"] for p in parts]
    return s


# ---------------------------------------------------------------------------------------
# named workloads: (Setup, config overrides)

def base_config(dt: float, steps: int, **over) -> dict:
    c = dict(dt=dt, timesteps=steps, modulo=max(1, steps // 10), enable_fracture=1, self_contact=1,
             nl_bdry_only=0, allow_damping=1, allow_friction=1, save_file=0)
    c.update(over)
    return c


def two_sphere(R=1.0 * MM, h=0.1 * MM, v=20.0, gap=0.2, seed=0, steps=2000, dt=1e-8, walls=False):
    """Config 0: sphere B moves at -v along x towards sphere A at rest; surface gap gap*h."""
    rng = np.random.default_rng(seed)
    Rc = 0.5 * h
    loc = lattice("sphere", 2 * R, h)
    A = make_particle(loc, h, GLASS, 3.0, rng, 0.05, (0, 0, 0), Rc=Rc)
    B = make_particle(loc, h, GLASS, 3.0, rng, 0.05, (2 * R + gap * h, 0, 0), vel=(-v, 0, 0), Rc=Rc)
    wall = None
    if walls:
        L = 3 * R
        wall = dict(allow=1, geom=[-1.5 * R, -1.02 * R, -1.02 * R, L + 0.5 * R, 1.02 * R, 1.02 * R])
    s = finish([A, B], Rc, dt, wall=wall)
    s.meta["name"] = "two_sphere"
    return s, base_config(dt, steps)


def cubes125(n=5, edge=1.0 * MM, h=0.125 * MM, seed=1, steps=20000, dt=2e-8, g=9.81 * 1e4, gap=0.9 * MM):
    """Config 1: n^3 randomly rotated cubes in a walled box under scaled gravity."""
    rng = np.random.default_rng(seed)
    Rc = 0.5 * h
    loc = lattice("cube", edge, h)
    pitch = edge * math.sqrt(3) + gap * 0.2
    parts = []
    for iz in range(n):
        for iy in range(n):
            for ix in range(n):
                c = ((ix - (n - 1) / 2) * pitch, (iy - (n - 1) / 2) * pitch, (iz - (n - 1) / 2) * pitch)
                p = make_particle(loc, h, GLASS, 3.0, rng, 0.05, c, rotation=random_rotation(rng), Rc=Rc)
                npn = len(p["pos"])
                # gravity as extforce = rho*g (force density) and initial acc = g, the convention
                # of examples/3D-HPC-aggregate-particle-breakage/setup.py:135-152
                p["extforce"] = np.tile([0.0, 0.0, -g * p["rho"]], (npn, 1))
                p["acc"] = np.tile([0.0, 0.0, -g], (npn, 1))
                parts.append(p)
    half = n * pitch / 2 + 0.5 * Rc
    wall = dict(allow=1, geom=[-half, -half, -half, half, half, half + pitch])
    s = finish(parts, Rc, dt, wall=wall)
    s.meta["name"] = "cubes125"
    return s, base_config(dt, steps)


def notch_cut(pos: np.ndarray, conn: np.ndarray, x_wall: float, y0: float, y1: float, z0: float,
              z_extrusion: float) -> np.ndarray:
    """Removes the bonds whose segment crosses the notch face x = x_wall, y in [y0, y1],
    z in [z0, z0 + z_extrusion] (wall_line_intrsect, exp_dict.py:96-122: inclusive bounds)."""
    keep = np.ones(len(conn), dtype=bool)
    for a in range(0, len(conn), 1 << 22):
        c = conn[a:a + (1 << 22)].astype(np.int64)
        p6, p7 = pos[c[:, 0]], pos[c[:, 1]]
        x6, x7 = p6[:, 0], p7[:, 0]
        cross = (np.minimum(x6, x7) <= x_wall) & (x_wall <= np.maximum(x6, x7))
        idx = np.nonzero(cross)[0]
        if len(idx):
            dx = x7[idx] - x6[idx]
            with np.errstate(divide="ignore", invalid="ignore"):
                t = (x_wall - x6[idx]) / dx
            ip = p6[idx] + t[:, None] * (p7[idx] - p6[idx])
            hit = (y0 <= ip[:, 1]) & (ip[:, 1] <= y1) & (z0 <= ip[:, 2]) & (ip[:, 2] <= z0 + z_extrusion)
            keep[a + idx[hit]] = False
    return conn[keep]


def notched_plate(Lx=100.0 * MM, Ly=200.0 * MM, Lz=9.0 * MM, h=0.5 * MM, notch_len=50.0 * MM,
                  notch_w=1.5 * MM, notch_x=(25.0 * MM, 75.0 * MM), imp_w=50.0 * MM, imp_len=10.0 * MM, v=32.0,
                  seed=4, steps=5000, dt=2e-8, jitter=0.05, gap=0.2):
    """Config 3: a steel plate Lx x Ly x Lz with two edge notches of length notch_len and width
    notch_w running from the edge y = 0 at x = notch_x; bonds across the notch faces are cut
    like the reference's Kalthoff setup (exp_dict.py:1095-1163). A steel impactor block, imp_w
    wide and unbreakable, hits the notched edge between the notches at v along +y; the surface
    gap between them is gap*h."""
    rng = np.random.default_rng(seed)
    Rc = 0.5 * h

    def block(ex, ey, ez, origin):
        ax = [(np.arange(max(1, int(round(e / h)))) + 0.5) * h for e in (ex, ey, ez)]
        X, Y, Z = np.meshgrid(*ax, indexing="ij")
        P = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1) + np.asarray(origin)
        return P + rng.uniform(-jitter * h, jitter * h, size=P.shape)

    P = block(Lx, Ly, Lz, (0.0, 0.0, 0.0))
    inside = np.zeros(len(P), dtype=bool)
    for xc in notch_x:  # the notch slots carry no material
        inside |= (np.abs(P[:, 0] - xc) < 0.5 * notch_w) & (P[:, 1] < notch_len)
    P = P[~inside]
    delta = 3.0 * h
    conn = bonds(P, delta).astype(np.int64)
    for xc in notch_x:
        conn = notch_cut(P, conn, xc, -h, notch_len, -h, Lz + 2 * h)
    m = material_3d(STEEL, delta)
    plate = dict(pos=P, vol=np.full(len(P), h ** 3), conn=conn.astype(np.uint32), h=h, **m)
    x0 = 0.5 * (notch_x[0] + notch_x[1]) - 0.5 * imp_w
    # facing node layers (1 + gap) h apart, like two lattices whose surfaces are gap*h apart
    Q = block(imp_w, imp_len, Lz, (x0, -imp_len - gap * h, 0.0))
    imp = dict(pos=Q, vol=np.full(len(Q), h ** 3), conn=bonds(Q, delta), h=h,
               vel=np.tile([0.0, v, 0.0], (len(Q), 1)), breakable=0, **material_3d(STEEL, delta))
    s = finish([plate, imp], Rc, dt)
    s.meta["name"] = "notched_plate"
    return s, base_config(dt, steps)


def _grid_pack(rng, m: int, count: int, pitch: float, hs, smin: float, smax: float) -> list:
    """`count` particles of random shape/size/resolution on the first cells of an m^3 grid of
    pitch `pitch` centred on the origin (cells in z, y, x order)."""
    parts = []
    box = m * pitch
    for idx in range(count):
        iz, rem = divmod(idx, m * m)
        iy, ix = divmod(rem, m)
        kind = ("sphere", "cube", "ellipsoid")[int(rng.integers(3))]
        h = float(hs[int(rng.integers(len(hs)))])
        # sizes are bounding diameters, so that randomly rotated particles on the
        # 1.5 mm pitch never overlap: a cube of size d has edge d / sqrt(3)
        if kind == "ellipsoid":
            size = rng.uniform(smin, smax, size=3)
        elif kind == "cube":
            size = float(rng.uniform(smin, smax)) / math.sqrt(3.0)
        else:
            size = float(rng.uniform(smin, smax))
        loc = lattice(kind, size, h)
        c = np.array([(ix + 0.5) * pitch, (iy + 0.5) * pitch, (iz + 0.5) * pitch]) - box / 2
        c = c + rng.uniform(-0.02, 0.02, size=3) * pitch
        p = make_particle(loc, h, GLASS, 3.0, rng, 0.05, c, rotation=random_rotation(rng), Rc=None)
        parts.append(p)
    return parts


def crush512(n=8, box=12.0 * MM, seed=2, steps=10000, dt=5e-9, hs=(0.05 * MM, 0.075 * MM, 0.1 * MM),
             smin=0.6 * MM, smax=1.4 * MM, wall_speed=-1.0, count=None):
    """Config 2: n^3 particles of random shape/size/resolution in a box; top wall moves down.
    count: only the first `count` particles of the same packing (the contact stiffness is the
    whole packing's, whose largest nodal volume is max(hs)^3)."""
    rng = np.random.default_rng(seed)
    Rc = 0.5 * min(hs)
    parts = _grid_pack(rng, n, n ** 3 if count is None else min(int(count), n ** 3), box / n, hs, smin, smax)
    half = box / 2
    wall = dict(allow=1, geom=[-half, -half, -half, half, half, half])
    kn = None if count is None else stable_kn(kn_rule(Rc), GLASS["rho"], max(hs) ** 3, dt)
    s = finish(parts, Rc, dt, wall=wall, kn=kn)
    s.meta["name"] = "crush512"
    return s, base_config(dt, steps, speed_wall_z_max=wall_speed)


def crush512_4m(steps=10000, count=None):
    """Config 2 at the node count quoted beside it (~4 M nodes, ~3.5e8 directed bonds): the same
    512-particle packing with every lattice spacing scaled by 0.6 (h from {0.03, 0.045, 0.06}
    mm) and dt lowered to 3e-9 s, below the bond-based critical step delta*sqrt(rho/(18 K))
    of the finest lattice (4.8e-9 s at h = 0.03 mm)."""
    s, cfg = crush512(steps=steps, dt=3e-9, hs=(0.03 * MM, 0.045 * MM, 0.06 * MM), count=count)
    s.meta["name"] = "crush512_4m"
    return s, cfg


def crush_contact(count=16, steps=2000, box=9.6 * MM, wall_speed=-20.0):
    """Config 2's particle mix in contact and breaking from the first steps: the first `count`
    particles of crush512_4m's packing (spheres, cubes and ellipsoids at h = 0.03, 0.045 and
    0.06 mm, dt = 3e-9 s) drawn on a 1.2 mm pitch (box 9.6 mm) instead of 1.5 mm, so that
    neighbours touch, with the top wall started at the top of the packing and moving down at
    |wall_speed|."""
    s, cfg = crush512(n=8, box=box, steps=steps, dt=3e-9, hs=(0.03 * MM, 0.045 * MM, 0.06 * MM), count=count)
    cfg.update(wall_z_max=float(s.pos[:, 2].max()) + 0.01 * MM, speed_wall_z_max=wall_speed, compute_wall_reaction=1)
    s.meta["name"] = "crush_contact"
    return s, cfg


def aggregate(n_particles: int, seed: int, steps: int, wall_speed: float = -1.0, dt=5e-9, pitch=1.5 * MM,
              hs=(0.05 * MM, 0.075 * MM, 0.1 * MM), smin=0.6 * MM, smax=1.4 * MM):
    """One aggregate of the serving stream: n_particles drawn like config 2's particles, packed
    on the smallest cubic grid of config 2's pitch that holds them, in a walled box whose top
    wall moves down at |wall_speed|."""
    rng = np.random.default_rng(seed)
    Rc = 0.5 * min(hs)
    m = 1
    while m ** 3 < n_particles:
        m += 1
    parts = _grid_pack(rng, m, n_particles, pitch, hs, smin, smax)
    half = m * pitch / 2
    wall = dict(allow=1, geom=[-half, -half, -half, half, half, half])
    s = finish(parts, Rc, dt, wall=wall)
    s.meta["name"] = f"aggregate{n_particles}"
    return s, base_config(dt, steps, speed_wall_z_max=-abs(wall_speed))


def serving_stream(n: int = 256, rate: float = 4.0, seed: int = 3, pmin: int = 8, pmax: int = 64,
                   steps=(2000, 10000), speed=(0.5, 2.0)) -> list[dict]:
    """Config 4's request stream: Poisson arrivals at `rate` per second; each request is an
    aggregate of pmin..pmax particles with a random compression speed and step count.
    Returns light specs; aggregate(**spec["gen"]) builds the setup."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += float(rng.exponential(1.0 / rate))
        npart = int(rng.integers(pmin, pmax + 1))
        nst = int(rng.integers(steps[0], steps[1] + 1))
        v = float(rng.uniform(speed[0], speed[1]))
        out.append(dict(rid=i, arrival=t, gen=dict(n_particles=npart, seed=int(seed * 100003 + i), steps=nst,
                                                   wall_speed=-v)))
    return out


WORKLOADS = {"two_sphere": two_sphere, "cubes125": cubes125, "crush512": crush512, "crush512_4m": crush512_4m,
             "notched_plate": notched_plate, "crush_contact": crush_contact}


def build_aggregate(kw: dict):
    """aggregate(**kw): a top-level function, so that a process pool can build requests."""
    return aggregate(**kw)
