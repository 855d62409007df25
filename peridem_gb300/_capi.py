"""ctypes binding of include/peridem_gb300.h (the engine's C-ABI).

The library is built in-tree (peridem_gb300/_lib/libperidem_gb300.so) by
peridem_gb300.build; loading fails loudly when it is missing: there is no fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_lib" / "libperidem_gb300.so"

PD_OK = 0
PD_EINVAL = -1
PD_ECUDA = -2
PD_ENOMEM = -3
PD_EIO = -4
PD_ETIMEOUT = -5
PD_EDEVICE = -6
PD_ECONFIG = -7
PD_ESTATE = -8
PD_DERR_STAGE_TIMEOUT = 8
PD_FP64 = 0
PD_FP32C = 1
PD_DERR_NONFINITE = 1
PD_DERR_CAND_OVERFLOW = 2

_u32, _i32, _u64, _f64 = C.c_uint32, C.c_int32, C.c_uint64, C.c_double


class PdConfig(C.Structure):
    """pd_config: the main.conf fields of ConfigVal (src/read/read_config.h:14-167)."""
    _fields_ = [
        ("timesteps", _u32), ("modulo", _u32), ("dt", _f64), ("is_parallel", _i32),
        ("do_resume", _i32), ("wall_resume", _i32), ("resume_ind", _u32), ("save_file", _i32),
        ("enable_fracture", _i32), ("nl_bdry_only", _i32), ("allow_damping", _i32),
        ("allow_friction", _i32), ("normal_stiffness", _f64), ("damping_ratio", _f64),
        ("friction_coefficient", _f64), ("new_snot", _f64), ("self_contact", _i32),
        ("self_contact_rad", _f64), ("enable_cohesion", _i32), ("cohesion_scaling", _f64),
        ("enable_torque", _i32), ("set_torque_timestep", _i32), ("set_fracture_timestep", _i32),
        ("set_self_contact_timestep", _i32), ("set_zero_wall_speed_timestep", _i32),
        ("set_damping_timestep", _i32), ("set_movable_index", _i32), ("set_movable_timestep", _i32),
        ("set_stoppable_index", _i32), ("set_stoppable_timestep", _i32), ("reset_partzero_y", _i32),
        ("reset_partzero_y_timestep", _u32), ("wheel_rad", _f64), ("particle_w_fixed_velocity", _i32),
        ("set_fix_velocity_timestep", _i32), ("fix_velocity_angular", _i32),
        ("prescribed_angular_vel", _f64), ("fix_velocity_mean_x", _i32),
        ("prescribed_velocity_mean_x", _f64), ("wall_left", _f64), ("wall_right", _f64),
        ("wall_top", _f64), ("wall_bottom", _f64), ("wall_x_min", _f64), ("wall_y_min", _f64),
        ("wall_z_min", _f64), ("wall_x_max", _f64), ("wall_y_max", _f64), ("wall_z_max", _f64),
        ("speed_wall_left", _f64), ("speed_wall_right", _f64), ("speed_wall_top", _f64),
        ("speed_wall_bottom", _f64), ("speed_wall_x_min", _f64), ("speed_wall_y_min", _f64),
        ("speed_wall_z_min", _f64), ("speed_wall_x_max", _f64), ("speed_wall_y_max", _f64),
        ("speed_wall_z_max", _f64), ("brazil", _i32), ("brazil_reset_wall_bottom_freq", _i32),
        ("brazil_nonzero_wall_bottom_speed_freq", _i32), ("brazil_reset_wall_bottom_y", _f64),
        ("forcefield_type", _i32), ("forcefield_scaling", _f64), ("gradient_extforce", _i32),
        ("extforce_maxstep", _u32), ("compute_wall_reaction", _i32),
        ("setup_filename", C.c_char * 1024), ("output_dir", C.c_char * 1024),
        ("n_unknown_keys", _u32),
    ]


class PdSetupArrays(C.Structure):
    _fields_ = [
        ("n_particles", _u32),
        ("node_offset", C.POINTER(_u64)), ("pos", C.POINTER(_f64)), ("vol", C.POINTER(_f64)),
        ("disp", C.POINTER(_f64)), ("vel", C.POINTER(_f64)), ("acc", C.POINTER(_f64)),
        ("extforce", C.POINTER(_f64)), ("conn_offset", C.POINTER(_u64)), ("conn", C.POINTER(_u32)),
        ("bdry_offset", C.POINTER(_u64)), ("bdry", C.POINTER(_u32)),
        ("clamped_offset", C.POINTER(_u64)), ("clamped", C.POINTER(_u32)),
        ("delta", C.POINTER(_f64)), ("rho", C.POINTER(_f64)), ("cnot", C.POINTER(_f64)),
        ("snot", C.POINTER(_f64)), ("torque_val", C.POINTER(_f64)),
        ("movable", C.POINTER(_i32)), ("breakable", C.POINTER(_i32)), ("stoppable", C.POINTER(_i32)),
        ("torque_axis", C.POINTER(_u32)),
        ("contact_radius", _f64), ("normal_stiffness", _f64), ("damping_ratio", _f64),
        ("friction_coefficient", _f64), ("allow_wall", _i32), ("n_geom_wall", _i32),
        ("geom_wall_info", _f64 * 6),
    ]


class PdStats(C.Structure):
    _fields_ = [("step", _u64), ("live_bonds", _u64), ("pairwise_computations", _u64),
                ("contacts", _u64), ("rebuilds", _u64), ("device_errors", _u32)]


# every entry point include/peridem_gb300.h declares: (name, restype, argtypes)
_P = C.c_void_p
SIGNATURES = [
    ("pd_config_default", C.c_int, [C.POINTER(PdConfig)]),
    ("pd_config_read", C.c_int, [C.c_char_p, C.POINTER(PdConfig)]),
    ("pd_create_from_arrays", C.c_int, [C.POINTER(PdSetupArrays), C.POINTER(PdConfig), C.c_int, C.POINTER(_P)]),
    ("pd_open", C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.POINTER(_P)]),
    ("pd_run", C.c_int, [_P]),
    ("pd_step", C.c_int, [_P, _u32]),
    ("pd_sync", C.c_int, [_P, C.c_int]),
    ("pd_set_stream", C.c_int, [_P, _P]),
    ("pd_num_nodes", C.c_int, [_P, C.POINTER(_u64), C.POINTER(_u32)]),
    ("pd_get_state", C.c_int, [_P, _P, _P, _P, _P]),
    ("pd_get_disp", C.c_int, [_P, _P]),
    ("pd_get_node_state", C.c_int, [_P, _P, _P, _P, _P, _P]),
    ("pd_get_applied_force_density", C.c_int, [_P, _P]),
    ("pd_get_damage", C.c_int, [_P, _P]),
    ("pd_get_sim_damage", C.c_int, [_P, _u32, _P]),
    ("pd_set_state", C.c_int, [_P, _P, _P, _P]),
    ("pd_get_connectivity", C.c_int, [_P, _u32, _P, _u64, C.POINTER(_u64)]),
    ("pd_get_wall", C.c_int, [_P, _P, _P]),
    ("pd_get_aabb", C.c_int, [_P, _P]),
    ("pd_get_stats", C.c_int, [_P, C.POINTER(PdStats)]),
    ("pd_write_frame", C.c_int, [_P, _u32]),
    ("pd_last_error", C.c_char_p, [_P]),
    ("pd_global_error", C.c_char_p, []),
    ("pd_close", C.c_int, [_P]),
    ("pd_set_tuning", C.c_int, [_P, _f64, _u32, C.c_int, C.c_int, C.c_int]),
    ("pd_clear_device_errors", C.c_int, [_P]),
    ("pd_step_bytes", _f64, [_P]),
    ("pd_profile_steps", C.c_int, [_P, _u32, _P]),
    ("pd_count_live_bonds", C.c_int, [_P, C.POINTER(_u64)]),
    ("pd_count_live_bonds_noalloc", C.c_int, [_P, C.POINTER(_u64)]),
    ("pd_autotune", C.c_int, [_P, _u32, C.POINTER(C.c_int), _P]),
    ("pd_set_variant", C.c_int, [_P, C.c_int]),
    ("pd_set_persist_lanes", C.c_int, [_P, C.c_int]),
    ("pd_persist_lanes", C.c_int, [_P]),
    ("pd_num_variants", C.c_int, []),
    ("pd_graph_mode", C.c_int, [_P]),
    ("pd_snapshot", C.c_int, [_P]),
    ("pd_restore", C.c_int, [_P]),
    ("pd_resume", C.c_int, [_P, _u32, C.c_int]),
    ("pd_files_error", C.c_char_p, []),
    ("pd_h5_writer_new", _P, []),
    ("pd_h5_writer_add", C.c_int, [_P, C.c_char_p, C.c_int, C.c_int, C.POINTER(_u64), _P]),
    ("pd_h5_writer_write", C.c_int, [_P, C.c_char_p]),
    ("pd_h5_writer_free", None, [_P]),
    ("pd_h5_open", _P, [C.c_char_p]),
    ("pd_h5_list", C.c_size_t, [_P, C.c_char_p, C.c_size_t]),
    ("pd_h5_info", C.c_int, [_P, C.c_char_p, C.POINTER(C.c_int), C.POINTER(_u64)]),
    ("pd_h5_read", C.c_int, [_P, C.c_char_p, C.c_int, _P, _u64]),
    ("pd_h5_close", None, [_P]),
    ("pd_create_batch", C.c_int, [C.POINTER(PdSetupArrays), C.POINTER(PdConfig), _u32, C.c_int, C.POINTER(_P)]),
    ("pd_estimate_bytes", C.c_int, [C.POINTER(PdSetupArrays), _u32, C.c_int, C.POINTER(_u64)]),
    ("pd_device_bytes", C.c_int, [_P, C.POINTER(_u64)]),
    ("pd_device_memory", C.c_int, [C.POINTER(_u64), C.POINTER(_u64)]),
    ("pd_num_sims", C.c_int, [_P, C.POINTER(_u32)]),
    ("pd_sim_range", C.c_int, [_P, _u32, C.POINTER(_u64), C.POINTER(_u64), C.POINTER(_u32), C.POINTER(_u32)]),
    ("pd_sim_steps", C.c_int, [_P, _u32, C.POINTER(_u64)]),
    ("pd_finish_sim", C.c_int, [_P, _u32]),
    ("pd_get_sim_state", C.c_int, [_P, _u32, _P, _P, _P, _P]),
    ("pd_get_sim_disp", C.c_int, [_P, _u32, _P]),
    ("pd_get_sim_wall", C.c_int, [_P, _u32, _P, _P]),
    ("pd_save_sim", C.c_int, [_P, _u32, _P, _u64, C.POINTER(_u64)]),
    ("pd_load_sim", C.c_int, [_P, _u32, _P, _u64]),
    ("pd_query_pairs", C.c_int, [_P, _P, _P, _u32, _P, _u64, _P]),
    ("pd_query_near", C.c_int, [_P, _P, _P, _u32, _P, _P]),
    ("pd_pairs_error", C.c_char_p, []),
]

_lib = None


def lib() -> C.CDLL:
    """Load the engine library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run peridem_gb300.build.build_engine() first")
        L = C.CDLL(str(LIB_PATH))
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class PdError(RuntimeError):
    def __init__(self, rc: int, msg: str):
        super().__init__(f"[{rc}] {msg}")
        self.rc = rc


def default_config(**over) -> PdConfig:
    cfg = PdConfig()
    lib().pd_config_default(C.byref(cfg))
    for k, v in over.items():
        if not hasattr(cfg, k):
            raise KeyError(k)
        setattr(cfg, k, v.encode() if isinstance(v, str) else v)
    return cfg


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _p(a, ctype):
    return None if a is None else a.ctypes.data_as(C.POINTER(ctype))


def setup_struct(s) -> tuple[PdSetupArrays, list]:
    """Fill a pd_setup_arrays from a peridem_gb300.setupdata.Setup; returns the struct and the
    list of arrays that must stay alive while it is used."""
    keep = []

    def a(x, dt):
        arr = np.ascontiguousarray(x, dtype=dt)
        keep.append(arr)
        return arr

    st = PdSetupArrays()
    st.n_particles = s.n_particles
    st.node_offset = _p(a(s.node_offset, np.uint64), _u64)
    st.pos = _p(a(s.pos, np.float64), _f64)
    st.vol = _p(a(s.vol, np.float64), _f64)
    st.disp = _p(a(s.disp, np.float64), _f64)
    st.vel = _p(a(s.vel, np.float64), _f64)
    st.acc = _p(a(s.acc, np.float64), _f64)
    st.extforce = _p(a(s.extforce, np.float64), _f64)
    st.conn_offset = _p(a(s.conn_offset, np.uint64), _u64)
    st.conn = _p(a(s.conn if len(s.conn) else np.zeros((1, 2)), np.uint32), _u32)
    if s.bdry_offset is not None:
        st.bdry_offset = _p(a(s.bdry_offset, np.uint64), _u64)
        st.bdry = _p(a(s.bdry if len(s.bdry) else np.zeros(1), np.uint32), _u32)
    if s.clamped_offset is not None:
        st.clamped_offset = _p(a(s.clamped_offset, np.uint64), _u64)
        st.clamped = _p(a(s.clamped if len(s.clamped) else np.zeros(1), np.uint32), _u32)
    st.delta = _p(a(s.delta, np.float64), _f64)
    st.rho = _p(a(s.rho, np.float64), _f64)
    st.cnot = _p(a(s.cnot, np.float64), _f64)
    st.snot = _p(a(s.snot, np.float64), _f64)
    st.torque_val = _p(a(s.torque_val, np.float64), _f64)
    st.movable = _p(a(s.movable, np.int32), _i32)
    st.breakable = _p(a(s.breakable, np.int32), _i32)
    st.stoppable = _p(a(s.stoppable, np.int32), _i32)
    st.torque_axis = _p(a(s.torque_axis, np.uint32), _u32)
    st.contact_radius = s.contact_radius
    st.normal_stiffness = s.normal_stiffness
    st.damping_ratio = s.damping_ratio
    st.friction_coefficient = s.friction_coefficient
    st.allow_wall = int(s.allow_wall)
    st.n_geom_wall = 6 if s.geom_wall_info is not None else 1
    if s.geom_wall_info is not None:
        for k in range(6):
            st.geom_wall_info[k] = float(s.geom_wall_info[k])
    return st, keep
