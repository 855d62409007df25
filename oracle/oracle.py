"""TEST INFRASTRUCTURE: Python access to the CPU oracle (libpd_oracle.so, the restatement in
pd_oracle.cpp) and, where it was built here, to PeriDEM's own code compiled against the
stand-in headers (oracle/_ref/libpd_ref.so). Imported only by tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline legs; the product never imports it."""
from __future__ import annotations

import ctypes as C
import os
import tempfile
import threading
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "_build" / "libpd_oracle.so"
REF_LIB = HERE / "_ref" / "libpd_ref.so"

_P = C.c_void_p
_u32, _u64 = C.c_uint32, C.c_uint64


def _capi():
    """The ctypes structure layouts of include/peridem_gb300.h (pure Python: importing them maps
    no library; the oracle never loads the engine library)."""
    from peridem_gb300 import _capi
    return _capi


_olib = None


def oracle_lib() -> C.CDLL:
    global _olib
    if _olib is None:
        if not ORACLE_LIB.exists():
            raise RuntimeError(f"{ORACLE_LIB} missing: run `make -C oracle`")
        L = C.CDLL(str(ORACLE_LIB))
        capi = _capi()
        L.or_config_default.argtypes = [C.POINTER(capi.PdConfig)]
        L.or_create.restype = _P
        L.or_create.argtypes = [C.POINTER(capi.PdSetupArrays), C.POINTER(capi.PdConfig)]
        L.or_set_threads.argtypes = [_P, C.c_int]
        L.or_set_cell_search.argtypes = [_P, C.c_int]
        L.or_step.argtypes = [_P, _u32]
        L.or_get_state.argtypes = [_P, _P, _P, _P, _P]
        L.or_get_disp.argtypes = [_P, _P]
        L.or_get_afd.argtypes = [_P, _P]
        L.or_get_connectivity.argtypes = [_P, _u32, _P, _u64, C.POINTER(_u64)]
        L.or_get_wall.argtypes = [_P, _P, _P]
        L.or_get_aabb.argtypes = [_P, _P]
        L.or_get_counts.argtypes = [_P, _P]
        L.or_get_stretch.restype = _u64
        L.or_get_stretch.argtypes = [_P, _u32, _P, _u64]
        L.or_set_state.argtypes = [_P, _P, _P, _P]
        L.or_set_connectivity.argtypes = [_P, _u32, _P, _u64]
        L.or_destroy.argtypes = [_P]
        _olib = L
    return _olib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def default_config(**over):
    """pd_config with ConfigVal's defaults (from the oracle library) and the given fields set."""
    capi = _capi()
    cfg = capi.PdConfig()
    oracle_lib().or_config_default(C.byref(cfg))
    for k, v in over.items():
        if not hasattr(cfg, k):
            raise KeyError(k)
        setattr(cfg, k, v.encode() if isinstance(v, str) else v)
    return cfg


class Oracle:
    """The CPU restatement, one simulation (threads=1 is the exact, serial path). cell_search:
    contact visits only the node pairs within reach, in the reference's order (the same sums,
    bit for bit; for large cases, whose brute-force contact loops would take minutes)."""

    def __init__(self, setup, config=None, threads: int = 1, cell_search: bool = False):
        capi = _capi()
        self.setup = setup
        self.cfg = config if isinstance(config, capi.PdConfig) else default_config(**(config or {}))
        st, keep = capi.setup_struct(setup)
        L = oracle_lib()
        self.h = L.or_create(C.byref(st), C.byref(self.cfg))
        del keep
        if not self.h:
            raise RuntimeError("or_create failed")
        self.N = setup.n_nodes
        self.P = setup.n_particles
        if threads != 1:
            L.or_set_threads(self.h, int(threads))
        if cell_search:
            L.or_set_cell_search(self.h, 1)

    def close(self):
        if getattr(self, "h", None):
            oracle_lib().or_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, n: int = 1):
        oracle_lib().or_step(self.h, int(n))

    def state(self) -> dict:
        out = {k: np.empty((self.N, 3)) for k in ("curpos", "vel", "acc", "force", "disp")}
        L = oracle_lib()
        L.or_get_state(self.h, _ptr(out["curpos"]), _ptr(out["vel"]), _ptr(out["acc"]), _ptr(out["force"]))
        L.or_get_disp(self.h, _ptr(out["disp"]))
        return out

    def afd(self) -> np.ndarray:
        out = np.empty((self.N, 3))
        oracle_lib().or_get_afd(self.h, _ptr(out))
        return out

    def connectivity(self, p: int) -> np.ndarray:
        L = oracle_lib()
        n = _u64()
        L.or_get_connectivity(self.h, p, None, 0, C.byref(n))
        out = np.empty((n.value, 2), dtype=np.uint32)
        L.or_get_connectivity(self.h, p, _ptr(out), n.value, C.byref(n))
        return out

    def wall(self):
        w = np.empty(6)
        r = np.empty((6, 3))
        oracle_lib().or_get_wall(self.h, _ptr(w), _ptr(r))
        return w, r

    def aabb(self) -> np.ndarray:
        out = np.empty((self.P, 6))
        oracle_lib().or_get_aabb(self.h, _ptr(out))
        return out

    def counts(self) -> dict:
        c = np.zeros(4, dtype=np.uint64)
        oracle_lib().or_get_counts(self.h, _ptr(c))
        return dict(pairwise=int(c[0]), contacts=int(c[1]), live_bonds=int(c[2]), step=int(c[3]))

    def set_state(self, disp=None, vel=None, acc=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (disp, vel, acc)]
        oracle_lib().or_set_state(self.h, *(_ptr(a) for a in arrs))

    def set_connectivity(self, p: int, pairs):
        a = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1, 2)
        oracle_lib().or_set_connectivity(self.h, p, _ptr(a), len(a))

    def stretch(self, p: int) -> np.ndarray:
        L = oracle_lib()
        n = L.or_get_stretch(self.h, p, None, 0)
        out = np.empty(n)
        L.or_get_stretch(self.h, p, _ptr(out), n)
        return out


def total_neighbors(conn: np.ndarray, n: int) -> np.ndarray:
    """Bonds per node of an (m, 2) Connectivity, each pair counted at both ends, as float64
    (examples/3D-HPC-aggregate-particle-breakage/plot3d_timestep.py:95-105)."""
    deg = np.zeros(n)
    np.add.at(deg, np.asarray(conn, dtype=np.int64).ravel(), 1.0)
    return deg


def damage(setup, conns) -> np.ndarray:
    """Per-node damage of all particles in file order from their current Connectivity
    (conns[p], local pairs): (orig - now) / orig with orig from the setup's Connectivity
    (plot3d_timestep.py:108-117 and 156-166; 0/0 gives NaN as numpy does there)."""
    out = []
    for p in range(setup.n_particles):
        n = int(setup.node_offset[p + 1] - setup.node_offset[p])
        orig = total_neighbors(setup.conn[int(setup.conn_offset[p]):int(setup.conn_offset[p + 1])], n)
        now = total_neighbors(conns[p], n)
        with np.errstate(invalid="ignore", divide="ignore"):
            out.append((orig - now) / orig)
    return np.concatenate(out) if out else np.zeros(0)


# ------------------------------------------------------------------------------------------
# PeriDEM's own code (oracle/_ref), driven through its main() with an in-memory file store

SHIM_F64, SHIM_I32, SHIM_U32, SHIM_I64 = 1, 2, 3, 4
_rlib = None


def ref_available() -> bool:
    return REF_LIB.exists()


def ref_lib() -> C.CDLL:
    global _rlib
    if _rlib is None:
        if not REF_LIB.exists():
            raise RuntimeError(f"{REF_LIB} missing: run `make -C oracle ref` where the reference sources exist")
        L = C.CDLL(str(REF_LIB))
        L.h5mem_clear.argtypes = []
        L.h5mem_put.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.POINTER(_u64), _P]
        L.h5mem_info.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_int), C.POINTER(_u64)]
        L.h5mem_get.argtypes = [C.c_char_p, C.c_char_p, C.c_int, _P]
        L.h5mem_files.restype = C.c_size_t
        L.h5mem_files.argtypes = [C.c_char_p, C.c_size_t]
        L.pd_ref_run.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.c_char_p]
        _rlib = L
    return _rlib


def _put(file: str, path: str, arr: np.ndarray, lib=None):
    arr = np.asarray(arr)
    if arr.dtype.kind == "f":
        code, arr = SHIM_F64, np.ascontiguousarray(arr, dtype=np.float64)
    else:
        code, arr = SHIM_I64, np.ascontiguousarray(arr, dtype=np.int64)
    dims = (_u64 * max(1, arr.ndim))(*arr.shape)
    (lib or ref_lib()).h5mem_put(file.encode(), path.encode(), code, arr.ndim, dims, _ptr(arr) if arr.size else None)


def _get(file: str, path: str, dtype=np.float64) -> np.ndarray | None:
    L = ref_lib()
    t = C.c_int()
    dims = (_u64 * 8)()
    r = L.h5mem_info(file.encode(), path.encode(), C.byref(t), dims)
    if r < 0:
        return None
    shape = tuple(int(dims[i]) for i in range(r))
    code = SHIM_F64 if np.dtype(dtype).kind == "f" else SHIM_I64
    out = np.empty(shape, dtype=np.float64 if code == SHIM_F64 else np.int64)
    L.h5mem_get(file.encode(), path.encode(), code, _ptr(out))
    return out


def put_setup(file: str, s, lib=None) -> None:
    """Write a Setup into the in-memory store in the dataset layout exp_dict.py:2119-2185 writes
    (h5py stores Python ints as int64 and scalars as (1,1) datasets). lib: another library built
    with the stand-in HDF5 store (default: oracle/_ref/libpd_ref.so)."""
    for p in range(s.n_particles):
        g = "P_%05d" % p
        sl = s.particle_slice(p)
        n = sl.stop - sl.start
        _put(file, g + "/Pos", s.pos[sl], lib)
        _put(file, g + "/Vol", s.vol[sl].reshape(n, 1), lib)
        _put(file, g + "/Connectivity", s.particle_conn(p).astype(np.int64).reshape(-1, 2), lib)
        b = s.particle_list(s.bdry_offset, s.bdry, p)
        _put(file, g + "/bdry_nodes", np.asarray(b, np.int64).reshape(-1, 1), lib)
        cl = s.particle_list(s.clamped_offset, s.clamped, p)
        _put(file, g + "/clamped_nodes", np.asarray(cl, np.int64).reshape(-1), lib)
        for key, arr in (("disp", s.disp), ("vel", s.vel), ("acc", s.acc), ("extforce", s.extforce)):
            _put(file, g + "/" + key, arr[sl], lib)
        for key, arr in (("delta", s.delta), ("rho", s.rho), ("cnot", s.cnot), ("snot", s.snot),
                         ("torque_val", s.torque_val)):
            _put(file, g + "/" + key, np.array([[arr[p]]], dtype=np.float64), lib)
        for key, arr in (("torque_axis", s.torque_axis), ("movable", s.movable), ("breakable", s.breakable),
                         ("stoppable", s.stoppable)):
            _put(file, g + "/" + key, np.array([[int(arr[p])]], dtype=np.int64), lib)
    _put(file, "total_particles_univ", np.array([[s.n_particles]], dtype=np.int64), lib)
    _put(file, "pairwise/contact_radius", np.array([[s.contact_radius]]), lib)
    _put(file, "pairwise/normal_stiffness", np.array([[s.normal_stiffness]]), lib)
    _put(file, "pairwise/damping_ratio", np.array([[s.damping_ratio]]), lib)
    _put(file, "pairwise/friction_coefficient", np.array([[s.friction_coefficient]]), lib)
    _put(file, "wall/allow_wall", np.array([[int(s.allow_wall)]], dtype=np.int64), lib)
    g = s.geom_wall_info if s.geom_wall_info is not None else np.zeros(1)
    _put(file, "wall/geom_wall_info", np.asarray(g, dtype=np.float64).reshape(-1, 1), lib)


def write_conf(path: str, cfg: dict) -> None:
    with open(path, "w") as f:
        f.write("# written by the test harness\n")
        for k, v in cfg.items():
            f.write(f"{k} = {v!r}\n" if isinstance(v, float) else f"{k} = {v}\n")


def run_reference(s, cfg: dict, outdir: str = "mem_out", setup_key: str = "mem_setup.h5",
                  log: str | None = None, stack_mb: int = 1024) -> dict:
    """Run PeriDEM's main() on a Setup with a config dict (main.conf keys). Returns the frames
    it wrote: {counter: {"particles": [per-particle dicts], "wall": {...}}}."""
    L = ref_lib()
    L.h5mem_clear()
    put_setup(setup_key, s)
    with tempfile.TemporaryDirectory() as td:
        conf = os.path.join(td, "main.conf")
        write_conf(conf, cfg)
        argv = [b"simulate3d", b"-c", conf.encode(), b"-i", setup_key.encode(), b"-o", outdir.encode()]
        arr = (C.c_char_p * len(argv))(*argv)
        logp = (log or os.path.join(td, "ref.log")).encode()
        rc = [None]

        def run():
            rc[0] = L.pd_ref_run(len(argv), arr, logp)

        old = threading.stack_size()
        threading.stack_size(stack_mb * 1024 * 1024)
        try:
            th = threading.Thread(target=run)
            th.start()
            th.join()
        finally:
            threading.stack_size(old)
        if rc[0] != 0:
            raise RuntimeError(f"reference main() returned {rc[0]}")
    frames = {}
    buf = C.create_string_buffer(1 << 20)
    L.h5mem_files(buf, len(buf))
    names = [x for x in buf.value.decode().split("\n") if x]
    for name in names:
        base = name.rsplit("/", 1)[-1]
        if base.startswith("tc_") and base.endswith(".h5"):
            cnt = int(base[3:8])
            parts = []
            for p in range(s.n_particles):
                g = "P_%05d/" % p
                d = {k: _get(name, g + k) for k in ("CurrPos", "vel", "acc", "force")}
                afd = _get(name, g + "applied_force_density")
                if afd is not None:
                    d["applied_force_density"] = afd
                d["Connectivity"] = _get(name, g + "Connectivity", np.int64)
                parts.append(d)
            frames.setdefault(cnt, {})["particles"] = parts
        elif base.startswith("wall_") and base.endswith(".h5"):
            cnt = int(base[5:10])
            frames.setdefault(cnt, {})["wall"] = {"wall_info": _get(name, "wall_info"),
                                                 "reaction": _get(name, "reaction")}
        elif base == "plotinfo.h5":
            frames["plotinfo"] = {k: _get(name, k) for k in ("f_l_counter", "dimension", "dt", "modulo",
                                                             "wall/allow_wall", "wall/geom_wall_info")}
    return frames
