"""In-memory form of PeriDEM's setup schema (exp_dict.py:2119-2185, read by
src/read/load_hdf5.h:41-181): particles concatenated in file order with per-particle
offsets, plus the pairwise contact constants and the wall geometry."""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Setup:
    node_offset: np.ndarray            # (P+1,) uint64
    pos: np.ndarray                    # (N,3) f64
    vol: np.ndarray                    # (N,) f64
    disp: np.ndarray                   # (N,3)
    vel: np.ndarray                    # (N,3)
    acc: np.ndarray                    # (N,3)
    extforce: np.ndarray               # (N,3)
    conn_offset: np.ndarray            # (P+1,) uint64
    conn: np.ndarray                   # (M,2) uint32, particle-local, rows i<j sorted
    delta: np.ndarray                  # (P,)
    rho: np.ndarray
    cnot: np.ndarray
    snot: np.ndarray
    torque_val: np.ndarray
    movable: np.ndarray                # (P,) int32
    breakable: np.ndarray
    stoppable: np.ndarray
    torque_axis: np.ndarray            # (P,) uint32
    contact_radius: float
    normal_stiffness: float
    damping_ratio: float
    friction_coefficient: float
    allow_wall: int = 0
    geom_wall_info: np.ndarray | None = None  # (6,) x_min y_min z_min x_max y_max z_max
    bdry_offset: np.ndarray | None = None
    bdry: np.ndarray | None = None
    clamped_offset: np.ndarray | None = None
    clamped: np.ndarray | None = None
    meta: dict = field(default_factory=dict)

    @property
    def n_particles(self) -> int:
        return len(self.node_offset) - 1

    @property
    def n_nodes(self) -> int:
        return int(self.node_offset[-1])

    @property
    def n_bonds_directed(self) -> int:
        return 2 * int(self.conn_offset[-1])

    def particle_slice(self, p: int) -> slice:
        return slice(int(self.node_offset[p]), int(self.node_offset[p + 1]))

    def particle_conn(self, p: int) -> np.ndarray:
        return self.conn[int(self.conn_offset[p]):int(self.conn_offset[p + 1])]

    def particle_list(self, off, arr, p):
        if off is None:
            return np.zeros(0, dtype=np.uint32)
        return arr[int(off[p]):int(off[p + 1])]

    def subset(self, particles) -> "Setup":
        """A setup holding only the listed particles (same contact constants and walls)."""
        parts = []
        for p in particles:
            sl = self.particle_slice(p)
            parts.append(dict(pos=self.pos[sl], vol=self.vol[sl], disp=self.disp[sl], vel=self.vel[sl],
                              acc=self.acc[sl], extforce=self.extforce[sl], conn=self.particle_conn(p),
                              delta=self.delta[p], rho=self.rho[p], cnot=self.cnot[p], snot=self.snot[p],
                              torque_val=self.torque_val[p], movable=self.movable[p],
                              breakable=self.breakable[p], stoppable=self.stoppable[p],
                              torque_axis=self.torque_axis[p],
                              bdry=self.particle_list(self.bdry_offset, self.bdry, p),
                              clamped=self.particle_list(self.clamped_offset, self.clamped, p)))
        wall = dict(allow=self.allow_wall, geom=self.geom_wall_info) if self.geom_wall_info is not None else None
        s = concat(parts, dict(contact_radius=self.contact_radius, normal_stiffness=self.normal_stiffness,
                               damping_ratio=self.damping_ratio, friction_coefficient=self.friction_coefficient),
                   wall)
        s.meta = dict(self.meta, subset=list(map(int, particles)))
        return s

    def nbytes(self) -> int:
        """Bytes of the host arrays a caller hands to pd_create_from_arrays."""
        tot = 0
        for k in ("node_offset", "pos", "vol", "disp", "vel", "acc", "extforce", "conn_offset", "conn"):
            tot += getattr(self, k).nbytes
        return int(tot)

    def save_npz(self, path):
        d = {k: getattr(self, k) for k in ("node_offset", "pos", "vol", "disp", "vel", "acc", "extforce",
                                           "conn_offset", "conn", "delta", "rho", "cnot", "snot", "torque_val",
                                           "movable", "breakable", "stoppable", "torque_axis", "bdry_offset",
                                           "bdry", "clamped_offset", "clamped")}
        d["scalars"] = np.array([self.contact_radius, self.normal_stiffness, self.damping_ratio,
                                 self.friction_coefficient, float(self.allow_wall)])
        d["geom_wall_info"] = self.geom_wall_info if self.geom_wall_info is not None else np.zeros(0)
        np.savez(path, **d)

    @staticmethod
    def load_npz(path) -> "Setup":
        z = np.load(path)
        sc = z["scalars"]
        g = z["geom_wall_info"]
        return Setup(node_offset=z["node_offset"], pos=z["pos"], vol=z["vol"], disp=z["disp"], vel=z["vel"],
                     acc=z["acc"], extforce=z["extforce"], conn_offset=z["conn_offset"], conn=z["conn"],
                     delta=z["delta"], rho=z["rho"], cnot=z["cnot"], snot=z["snot"], torque_val=z["torque_val"],
                     movable=z["movable"], breakable=z["breakable"], stoppable=z["stoppable"],
                     torque_axis=z["torque_axis"], contact_radius=float(sc[0]), normal_stiffness=float(sc[1]),
                     damping_ratio=float(sc[2]), friction_coefficient=float(sc[3]), allow_wall=int(sc[4]),
                     geom_wall_info=g if len(g) else None, bdry_offset=z["bdry_offset"], bdry=z["bdry"],
                     clamped_offset=z["clamped_offset"], clamped=z["clamped"])


def concat(parts: list[dict], contact: dict, wall: dict | None) -> Setup:
    """Assemble particles (dicts with pos, vol, conn, material scalars, ...) into a Setup."""
    P = len(parts)
    nn = np.array([len(p["pos"]) for p in parts], dtype=np.uint64)
    node_offset = np.zeros(P + 1, dtype=np.uint64)
    node_offset[1:] = np.cumsum(nn)
    nc = np.array([len(p["conn"]) for p in parts], dtype=np.uint64)
    conn_offset = np.zeros(P + 1, dtype=np.uint64)
    conn_offset[1:] = np.cumsum(nc)

    def cat(key, shape_last=3):
        out = []
        for p in parts:
            n = len(p["pos"])
            v = p.get(key)
            if v is None:
                v = np.zeros((n, shape_last))
            out.append(np.asarray(v, dtype=np.float64).reshape(n, shape_last))
        return np.concatenate(out, axis=0)

    def lists(key):
        offs = np.zeros(P + 1, dtype=np.uint64)
        vals = []
        for i, p in enumerate(parts):
            v = np.asarray(p.get(key, []), dtype=np.uint32).reshape(-1)
            offs[i + 1] = offs[i] + len(v)
            vals.append(v)
        return offs, (np.concatenate(vals) if vals else np.zeros(0, np.uint32))

    bo, bl = lists("bdry")
    co, cl = lists("clamped")
    conn = np.concatenate([np.asarray(p["conn"], dtype=np.uint32).reshape(-1, 2) for p in parts], axis=0) \
        if int(nc.sum()) else np.zeros((0, 2), np.uint32)
    s = Setup(
        node_offset=node_offset,
        pos=cat("pos"), vol=cat("vol", 1).reshape(-1), disp=cat("disp"), vel=cat("vel"), acc=cat("acc"),
        extforce=cat("extforce"), conn_offset=conn_offset, conn=conn,
        delta=np.array([p["delta"] for p in parts], dtype=np.float64),
        rho=np.array([p["rho"] for p in parts], dtype=np.float64),
        cnot=np.array([p["cnot"] for p in parts], dtype=np.float64),
        snot=np.array([p["snot"] for p in parts], dtype=np.float64),
        torque_val=np.array([p.get("torque_val", 0.0) for p in parts], dtype=np.float64),
        movable=np.array([p.get("movable", 1) for p in parts], dtype=np.int32),
        breakable=np.array([p.get("breakable", 1) for p in parts], dtype=np.int32),
        stoppable=np.array([p.get("stoppable", 1) for p in parts], dtype=np.int32),
        torque_axis=np.array([p.get("torque_axis", 2) for p in parts], dtype=np.uint32),
        contact_radius=float(contact["contact_radius"]),
        normal_stiffness=float(contact["normal_stiffness"]),
        damping_ratio=float(contact["damping_ratio"]),
        friction_coefficient=float(contact["friction_coefficient"]),
        allow_wall=int(wall["allow"]) if wall else 0,
        geom_wall_info=np.asarray(wall["geom"], dtype=np.float64) if wall else None,
        bdry_offset=bo, bdry=bl, clamped_offset=co, clamped=cl,
    )
    return s
