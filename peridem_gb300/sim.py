"""Python handle over the C-ABI (include/peridem_gb300.h): the in-process counterpart of
run_timeloop<3> (src/particle/timeloop.h:231-965). Arrays are numpy, N*3 row vectors in
particle file order, like the reference's vector<Matrix<double,1,3>>."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from ._capi import PdError, PD_FP64, PD_FP32C, default_config, lib, ptr, setup_struct
from .setupdata import Setup

PRECISIONS = {"fp64": PD_FP64, "fp32c": PD_FP32C}


def make_config(over: dict | None = None) -> _capi.PdConfig:
    return default_config(**(over or {}))


class Sim:
    """One simulation resident on the GPU."""

    def __init__(self, setup: Setup, config: dict | _capi.PdConfig | None = None, precision: str = "fp64",
                 handle=None):
        self.setup = setup
        self.cfg = config if isinstance(config, _capi.PdConfig) else make_config(config)
        self.precision = precision
        L = lib()
        if handle is not None:
            self.h = handle
        else:
            st, keep = setup_struct(setup)
            h = C.c_void_p()
            rc = L.pd_create_from_arrays(C.byref(st), C.byref(self.cfg), PRECISIONS[precision], C.byref(h))
            del keep
            if rc != 0:
                raise PdError(rc, L.pd_global_error().decode())
            self.h = h
        n = C.c_uint64()
        p = C.c_uint32()
        L.pd_num_nodes(self.h, C.byref(n), C.byref(p))
        self.N = n.value
        self.P = p.value

    # -- lifecycle ------------------------------------------------------------------------
    def _ck(self, rc: int):
        if rc != 0:
            raise PdError(rc, lib().pd_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            lib().pd_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- stepping --------------------------------------------------------------------------
    def step(self, n: int = 1, sync: bool = True, timeout_ms: int = -1):
        self._ck(lib().pd_step(self.h, int(n)))
        if sync:
            self.sync(timeout_ms)

    def sync(self, timeout_ms: int = -1):
        self._ck(lib().pd_sync(self.h, int(timeout_ms)))

    def set_stream(self, stream_ptr: int | None):
        self._ck(lib().pd_set_stream(self.h, C.c_void_p(stream_ptr) if stream_ptr else None))

    def tune(self, skin_frac: float = 0.0, cand_cap: int = 0, tpb: int = 0, stats: int = -1, graphs: int = -1):
        self._ck(lib().pd_set_tuning(self.h, float(skin_frac), int(cand_cap), int(tpb), int(stats), int(graphs)))

    # -- state -----------------------------------------------------------------------------
    def state(self) -> dict:
        out = {k: np.empty((self.N, 3)) for k in ("curpos", "vel", "acc", "force", "disp")}
        self._ck(lib().pd_get_node_state(self.h, ptr(out["curpos"]), ptr(out["vel"]), ptr(out["acc"]),
                                         ptr(out["force"]), ptr(out["disp"])))
        return out

    def applied_force_density(self) -> np.ndarray:
        out = np.empty((self.N, 3))
        self._ck(lib().pd_get_applied_force_density(self.h, ptr(out)))
        return out

    def damage(self) -> np.ndarray:
        """Per-node damage (N,), file order: the field plot3d_timestep.py:156-166 derives
        from a saved Connectivity (NaN for a node without bonds in the setup)."""
        out = np.empty(self.N)
        self._ck(lib().pd_get_damage(self.h, ptr(out)))
        return out

    def set_state(self, disp=None, vel=None, acc=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (disp, vel, acc)]
        self._ck(lib().pd_set_state(self.h, *(ptr(a) for a in arrs)))

    def connectivity(self, p: int) -> np.ndarray:
        n = C.c_uint64()
        self._ck(lib().pd_get_connectivity(self.h, p, None, 0, C.byref(n)))
        out = np.empty((n.value, 2), dtype=np.uint32)
        self._ck(lib().pd_get_connectivity(self.h, p, ptr(out), n.value, C.byref(n)))
        return out

    def wall(self) -> tuple[np.ndarray, np.ndarray]:
        w = np.empty(6)
        r = np.empty((6, 3))
        self._ck(lib().pd_get_wall(self.h, ptr(w), ptr(r)))
        return w, r

    def aabb(self) -> np.ndarray:
        out = np.empty((self.P, 6))
        self._ck(lib().pd_get_aabb(self.h, ptr(out)))
        return out

    def stats(self) -> dict:
        s = _capi.PdStats()
        self._ck(lib().pd_get_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}

    def step_bytes(self) -> float:
        return float(lib().pd_step_bytes(self.h))

    def profile(self, nsteps: int) -> np.ndarray:
        """Device ms per phase summed over nsteps real steps:
        [predictor, broad phase, fused force+corrector, end of step]."""
        out = np.zeros(4)
        self._ck(lib().pd_profile_steps(self.h, int(nsteps), ptr(out)))
        return out

    def autotune(self, steps_per_variant: int = 8) -> tuple[int, np.ndarray]:
        """Times every bond-kernel variant on the live state (restored afterwards) and keeps the
        fastest, then the launch modes and, where the contact candidate lists were rebuilt while
        stepping, wider contact skins. Returns (chosen variant, ms per step of each variant)."""
        nv = lib().pd_num_variants()
        ms = np.zeros(nv)
        ch = C.c_int()
        self._ck(lib().pd_autotune(self.h, int(steps_per_variant), C.byref(ch), ptr(ms)))
        return ch.value, ms

    def set_variant(self, v: int):
        self._ck(lib().pd_set_variant(self.h, int(v)))

    def graph_mode(self) -> int:
        """0 separate launches, 1 step graph, 2 step graph with a conditional broad phase,
        3 persistent launches."""
        return int(lib().pd_graph_mode(self.h))

    def set_persist_lanes(self, lanes: int):
        """Lanes per node of the persistent step's bond phase (0: by size)."""
        self._ck(lib().pd_set_persist_lanes(self.h, int(lanes)))

    def persist_lanes(self) -> int:
        return int(lib().pd_persist_lanes(self.h))

    def snapshot(self):
        self._ck(lib().pd_snapshot(self.h))

    def restore(self):
        self._ck(lib().pd_restore(self.h))

    def save_sim(self, i: int = 0) -> bytes:
        """Checkpoint of simulation i at the current step boundary (pd_save_sim): host bytes
        that pd_load_sim turns back into the same simulation, in this or another handle."""
        n = C.c_uint64()
        L = lib()
        rc = L.pd_save_sim(self.h, i, None, 0, C.byref(n))
        if rc != 0:
            raise PdError(rc, L.pd_global_error().decode())
        buf = C.create_string_buffer(n.value)
        rc = L.pd_save_sim(self.h, i, buf, n.value, C.byref(n))
        if rc != 0:
            raise PdError(rc, L.pd_global_error().decode())
        return buf.raw[:n.value]

    def load_sim(self, blob: bytes, i: int = 0):
        """Continues simulation i from a checkpoint of the same setup and config."""
        L = lib()
        rc = L.pd_load_sim(self.h, i, blob, len(blob))
        if rc != 0:
            raise PdError(rc, L.pd_global_error().decode())

    def live_bonds(self) -> int:
        n = C.c_uint64()
        self._ck(lib().pd_count_live_bonds(self.h, C.byref(n)))
        return int(n.value)


def _setup_array(setups):
    arr = (_capi.PdSetupArrays * len(setups))()
    keep = []
    for i, s in enumerate(setups):
        st, k = setup_struct(s)
        arr[i] = st
        keep.append(k)
    return arr, keep


def estimate_bytes(setups: list[Setup], precision: str = "fp32c") -> int:
    """Device bytes a batch of these setups would take (no device work)."""
    arr, keep = _setup_array(setups)
    b = C.c_uint64()
    rc = lib().pd_estimate_bytes(arr, len(setups), PRECISIONS[precision], C.byref(b))
    del keep
    if rc != 0:
        raise PdError(rc, lib().pd_global_error().decode())
    return int(b.value)


def device_memory() -> tuple[int, int]:
    """(free, total) bytes of the current device."""
    f, t = C.c_uint64(), C.c_uint64()
    rc = lib().pd_device_memory(C.byref(f), C.byref(t))
    if rc != 0:
        raise PdError(rc, lib().pd_global_error().decode())
    return int(f.value), int(t.value)


class Batch(Sim):
    """Independent simulations in one handle: every phase of a step is one launch over all of
    them. Simulation i keeps its own node order; finish(i) ends it at the current step."""

    def __init__(self, setups: list[Setup], configs: list, precision: str = "fp32c"):
        cfgs = (_capi.PdConfig * len(setups))()
        for i, c in enumerate(configs):
            cfgs[i] = c if isinstance(c, _capi.PdConfig) else make_config(c)
        arr, keep = _setup_array(setups)
        h = C.c_void_p()
        rc = lib().pd_create_batch(arr, cfgs, len(setups), PRECISIONS[precision], C.byref(h))
        del keep
        if rc != 0:
            raise PdError(rc, lib().pd_global_error().decode())
        self.setups = list(setups)
        super().__init__(setups[0], cfgs[0], precision, handle=h)
        self.n_sims = len(setups)

    def _gk(self, rc: int):
        if rc != 0:
            raise PdError(rc, lib().pd_global_error().decode() or lib().pd_last_error(self.h).decode())

    def poll(self) -> bool:
        """True when the handle's queued work is done (never blocks)."""
        rc = lib().pd_sync(self.h, 0)
        if rc == _capi.PD_ETIMEOUT:
            return False
        self._ck(rc)
        return True

    def sim_range(self, i: int) -> tuple[int, int, int, int]:
        n0, nn, p0, npp = C.c_uint64(), C.c_uint64(), C.c_uint32(), C.c_uint32()
        self._gk(lib().pd_sim_range(self.h, i, C.byref(n0), C.byref(nn), C.byref(p0), C.byref(npp)))
        return n0.value, nn.value, p0.value, npp.value

    def sim_steps(self, i: int) -> int:
        n = C.c_uint64()
        self._gk(lib().pd_sim_steps(self.h, i, C.byref(n)))
        return int(n.value)

    def finish(self, i: int):
        self._ck(lib().pd_finish_sim(self.h, i))

    def sim_state(self, i: int) -> dict:
        nn = self.sim_range(i)[1]
        out = {k: np.empty((nn, 3)) for k in ("curpos", "vel", "acc", "force", "disp")}
        self._ck(lib().pd_get_sim_state(self.h, i, ptr(out["curpos"]), ptr(out["vel"]), ptr(out["acc"]),
                                        ptr(out["force"])))
        self._ck(lib().pd_get_sim_disp(self.h, i, ptr(out["disp"])))
        return out

    def sim_damage(self, i: int) -> np.ndarray:
        out = np.empty(self.sim_range(i)[1])
        self._ck(lib().pd_get_sim_damage(self.h, i, ptr(out)))
        return out

    def sim_wall(self, i: int) -> tuple[np.ndarray, np.ndarray]:
        w = np.empty(6)
        r = np.empty((6, 3))
        self._ck(lib().pd_get_sim_wall(self.h, i, ptr(w), ptr(r)))
        return w, r

    def sim_connectivity(self, i: int, p: int) -> np.ndarray:
        return self.connectivity(self.sim_range(i)[2] + p)

    def device_bytes(self) -> int:
        b = C.c_uint64()
        self._gk(lib().pd_device_bytes(self.h, C.byref(b)))
        return int(b.value)
