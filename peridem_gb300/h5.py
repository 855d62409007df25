"""HDF5 files of PeriDEM's schema through the library's own reader/writer (no h5py needed).

write_setup() lays a Setup out the way exp_dict.Experiment.save does (exp_dict.py:2119-2185);
read_setup() reads it back like load_particles/load_contact/load_wall (load_hdf5.h:41-181);
read_frame() reads a tc_%05u.h5 / wall_%05u.h5 pair written by pd_write_frame.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._capi import lib
from .setupdata import Setup

F64, I32, U32, I64, U64, F32 = 1, 2, 3, 4, 5, 6
_NP = {F64: np.float64, I32: np.int32, U32: np.uint32, I64: np.int64, U64: np.uint64, F32: np.float32}


def _sig():
    L = lib()
    if getattr(L, "_h5_ready", False):
        return L
    P = C.c_void_p
    L.pd_h5_writer_new.restype = P
    L.pd_h5_writer_add.argtypes = [P, C.c_char_p, C.c_int, C.c_int, C.POINTER(C.c_uint64), P]
    L.pd_h5_writer_write.argtypes = [P, C.c_char_p]
    L.pd_h5_writer_free.argtypes = [P]
    L.pd_h5_open.restype = P
    L.pd_h5_open.argtypes = [C.c_char_p]
    L.pd_h5_list.restype = C.c_size_t
    L.pd_h5_list.argtypes = [P, C.c_char_p, C.c_size_t]
    L.pd_h5_info.argtypes = [P, C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_uint64)]
    L.pd_h5_read.argtypes = [P, C.c_char_p, C.c_int, P, C.c_uint64]
    L.pd_h5_close.argtypes = [P]
    L.pd_files_error.restype = C.c_char_p
    L._h5_ready = True
    return L


class Writer:
    def __init__(self):
        self.L = _sig()
        self.h = self.L.pd_h5_writer_new()
        self._keep = []

    def add(self, path: str, arr, dtype: int | None = None):
        a = np.asarray(arr)
        if dtype is None:
            dtype = F64 if a.dtype.kind == "f" else (I64 if a.dtype.kind == "i" else U64 if a.dtype.itemsize == 8 else U32)
        a = np.ascontiguousarray(a, dtype=_NP[dtype])
        dims = (C.c_uint64 * max(1, a.ndim))(*a.shape)
        self._keep.append(a)
        rc = self.L.pd_h5_writer_add(self.h, path.encode(), dtype, a.ndim, dims, a.ctypes.data_as(C.c_void_p))
        if rc != 0:
            raise RuntimeError(f"pd_h5_writer_add({path}) = {rc}")

    def write(self, filename: str):
        rc = self.L.pd_h5_writer_write(self.h, str(filename).encode())
        if rc != 0:
            raise OSError(self.L.pd_files_error().decode())

    def __del__(self):
        try:
            self.L.pd_h5_writer_free(self.h)
        except Exception:
            pass


class Reader:
    def __init__(self, filename):
        self.L = _sig()
        self.h = self.L.pd_h5_open(str(filename).encode())
        if not self.h:
            raise OSError(self.L.pd_files_error().decode())

    def paths(self) -> list[str]:
        n = self.L.pd_h5_list(self.h, None, 0)
        buf = C.create_string_buffer(n)
        self.L.pd_h5_list(self.h, buf, n)
        return [p for p in buf.value.decode().split("\n") if p]

    def read(self, path: str, dtype: int = F64) -> np.ndarray:
        rank = C.c_int()
        dims = (C.c_uint64 * 8)()
        if self.L.pd_h5_info(self.h, path.encode(), C.byref(rank), dims) != 0:
            raise KeyError(path)
        shape = tuple(int(dims[i]) for i in range(rank.value))
        out = np.empty(shape, dtype=_NP[dtype])
        if self.L.pd_h5_read(self.h, path.encode(), dtype, out.ctypes.data_as(C.c_void_p), out.nbytes) != 0:
            raise OSError(self.L.pd_files_error().decode())
        return out

    def has(self, path: str) -> bool:
        rank = C.c_int()
        dims = (C.c_uint64 * 8)()
        return self.L.pd_h5_info(self.h, path.lstrip("/").encode(), C.byref(rank), dims) == 0

    def close(self):
        if self.h:
            self.L.pd_h5_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def write_setup(filename, s: Setup):
    w = Writer()
    for p in range(s.n_particles):
        g = "P_%05d/" % p
        sl = s.particle_slice(p)
        n = sl.stop - sl.start
        w.add(g + "Pos", s.pos[sl])
        w.add(g + "Vol", s.vol[sl].reshape(n, 1))
        w.add(g + "Connectivity", s.particle_conn(p).astype(np.int64).reshape(-1, 2))
        w.add(g + "bdry_nodes", np.asarray(s.particle_list(s.bdry_offset, s.bdry, p), np.int64).reshape(-1, 1))
        w.add(g + "clamped_nodes", np.asarray(s.particle_list(s.clamped_offset, s.clamped, p), np.int64).reshape(-1))
        for key, arr in (("disp", s.disp), ("vel", s.vel), ("acc", s.acc), ("extforce", s.extforce)):
            w.add(g + key, arr[sl])
        for key, arr in (("delta", s.delta), ("rho", s.rho), ("cnot", s.cnot), ("snot", s.snot),
                         ("torque_val", s.torque_val)):
            w.add(g + key, np.array([[arr[p]]], dtype=np.float64))
        for key, arr in (("torque_axis", s.torque_axis), ("movable", s.movable), ("breakable", s.breakable),
                         ("stoppable", s.stoppable)):
            w.add(g + key, np.array([[int(arr[p])]], dtype=np.int64))
    w.add("total_particles_univ", np.array([[s.n_particles]], dtype=np.int64))
    for key, val in (("contact_radius", s.contact_radius), ("normal_stiffness", s.normal_stiffness),
                     ("damping_ratio", s.damping_ratio), ("friction_coefficient", s.friction_coefficient)):
        w.add("pairwise/" + key, np.array([[val]], dtype=np.float64))
    w.add("wall/allow_wall", np.array([[int(s.allow_wall)]], dtype=np.int64))
    g = s.geom_wall_info if s.geom_wall_info is not None else np.zeros(1)
    w.add("wall/geom_wall_info", np.asarray(g, dtype=np.float64).reshape(-1, 1))
    w.write(filename)


def read_setup(filename) -> Setup:
    from .setupdata import concat
    r = Reader(filename)
    P = int(r.read("total_particles_univ", I64).ravel()[0])
    parts = []
    for p in range(P):
        g = "P_%05d/" % p
        d = dict(pos=r.read(g + "Pos"), vol=r.read(g + "Vol").reshape(-1), conn=r.read(g + "Connectivity", U32),
                 disp=r.read(g + "disp"), vel=r.read(g + "vel"), acc=r.read(g + "acc"),
                 extforce=r.read(g + "extforce"))
        for k in ("delta", "rho", "cnot", "snot", "torque_val"):
            d[k] = float(r.read(g + k).ravel()[0])
        for k in ("torque_axis", "movable", "breakable", "stoppable"):
            d[k] = int(r.read(g + k, I64).ravel()[0])
        d["bdry"] = r.read(g + "bdry_nodes", U32).reshape(-1) if r.has(g + "bdry_nodes") else []
        d["clamped"] = r.read(g + "clamped_nodes", U32).reshape(-1) if r.has(g + "clamped_nodes") else []
        parts.append(d)
    contact = {k: float(r.read("pairwise/" + k).ravel()[0])
               for k in ("contact_radius", "normal_stiffness", "damping_ratio", "friction_coefficient")}
    gw = r.read("wall/geom_wall_info").reshape(-1)
    wall = dict(allow=int(r.read("wall/allow_wall", I64).ravel()[0]), geom=gw) if len(gw) == 6 else None
    return concat(parts, contact, wall)


def read_frame(outdir, counter: int, n_particles: int) -> dict:
    r = Reader(f"{outdir}/tc_{counter:05d}.h5")
    parts = []
    for p in range(n_particles):
        g = "P_%05d/" % p
        d = {k: r.read(g + k) for k in ("CurrPos", "vel", "acc", "force")}
        d["Connectivity"] = r.read(g + "Connectivity", U32)
        if r.has(g + "applied_force_density"):
            d["applied_force_density"] = r.read(g + "applied_force_density")
        parts.append(d)
    w = Reader(f"{outdir}/wall_{counter:05d}.h5")
    wall = {"wall_info": w.read("wall_info").reshape(-1)}
    if w.has("reaction"):
        wall["reaction"] = w.read("reaction")
    return {"particles": parts, "wall": wall}
