"""Boundary checks that need no GPU: the C-ABI library loads and exports every function the
public header declares; the main.conf grammar (src/read/read_config.h:170-435); the HDF5
setup/frame files of the schema."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from peridem_gb300 import _capi, h5
from tests import cases

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for hdr in (ROOT / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", hdr.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ \t\*]*?\b(pd_[A-Za-z0-9_]+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    L = _capi.lib()
    names = declared_functions()
    assert len(names) > 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    bound = {n for n, _, _ in _capi.SIGNATURES}
    assert not (bound - set(names)), bound - set(names)


def test_config_defaults_match_configval():
    c = _capi.default_config()
    assert c.timesteps == 8000 and c.modulo == 100 and c.dt == 0.02 / 1e5
    assert c.self_contact == 1 and c.enable_fracture == 0 and c.save_file == 1 and c.resume_ind == 50
    assert c.normal_stiffness == -1 and c.damping_ratio == -1 and c.new_snot == -1
    assert c.wall_top == -999 and c.wall_z_max == -999 and c.speed_wall_z_max == 0
    assert c.forcefield_scaling == 1e9 and c.set_movable_index == -1
    assert c.setup_filename == b"data/hdf5/all.h5" and c.output_dir == b"output/hdf5/"


def _parse(text, tmp_path, capfd=None):
    p = tmp_path / "main.conf"
    p.write_text(text)
    c = _capi.default_config()
    rc = _capi.lib().pd_config_read(str(p).encode(), C.byref(c))
    return rc, c


def test_config_grammar(tmp_path, capfd):
    rc, c = _parse("""# comment
timesteps = 1234
modulo=7
  dt =  2.5e-8   # whitespace anywhere
enable_fracture = 2
save_file = 0
speed_wall_z_max = -1
wall_top = 0.012
normal_stiffness = 5
self_contact = 0
#timesteps = 99
not_a_key = 3
speed_wall_top = -1
""", tmp_path)
    assert rc == 0
    assert c.timesteps == 1234 and c.modulo == 7 and c.dt == 2.5e-8
    assert c.enable_fracture == 1          # bool = stoi(value) != 0
    assert c.save_file == 0 and c.self_contact == 0
    assert c.speed_wall_z_max == -1.0 and c.wall_top == 0.012 and c.normal_stiffness == 5.0
    assert c.speed_wall_top == -1.0
    assert c.n_unknown_keys == 1
    err = capfd.readouterr().err
    assert "[Error]: Wrong config name: not_a_key !!" in err


def test_config_stoi_prefix_semantics(tmp_path):
    rc, c = _parse("timesteps = 100abc\nmodulo = 1e5\n", tmp_path)
    assert rc == 0 and c.timesteps == 100 and c.modulo == 1  # std::stoi stops at the first non-digit


def test_config_bad_value_is_an_error_not_an_abort(tmp_path):
    rc, c = _parse("timesteps = abc\n", tmp_path)
    assert rc == _capi.PD_ECONFIG


def test_config_missing_file(tmp_path):
    c = _capi.default_config()
    rc = _capi.lib().pd_config_read(str(tmp_path / "nope.conf").encode(), C.byref(c))
    assert rc == _capi.PD_ECONFIG and c.timesteps == 8000


def test_h5_setup_round_trip(tmp_path):
    s, cfg = cases.toggles()
    f = tmp_path / "setup.h5"
    h5.write_setup(f, s)
    raw = f.read_bytes()
    assert raw[:8] == b"\x89HDF\r\n\x1a\n" and raw[8] == 0  # superblock version 0
    s2 = h5.read_setup(f)
    for k in ("node_offset", "pos", "vol", "disp", "vel", "acc", "extforce", "conn_offset", "conn", "delta", "rho",
              "cnot", "snot", "torque_val", "movable", "breakable", "stoppable", "torque_axis", "bdry_offset",
              "bdry", "clamped_offset", "clamped"):
        np.testing.assert_array_equal(np.asarray(getattr(s, k), dtype=np.float64),
                                      np.asarray(getattr(s2, k), dtype=np.float64), err_msg=k)
    assert s2.normal_stiffness == s.normal_stiffness and s2.allow_wall == s.allow_wall
    np.testing.assert_array_equal(s2.geom_wall_info, s.geom_wall_info)


def test_h5_types_and_shapes(tmp_path):
    w = h5.Writer()
    w.add("a/b/c", np.arange(12, dtype=np.float64).reshape(4, 3))
    w.add("a/i32", np.array([[-3]], dtype=np.int32), h5.I32)
    w.add("u", np.array([1, 2, 3], dtype=np.uint32), h5.U32)
    w.add("empty", np.zeros((0,), dtype=np.int64))
    w.add("f32", np.array([1.5, -2.25], dtype=np.float32), h5.F32)
    f = tmp_path / "x.h5"
    w.write(f)
    r = h5.Reader(f)
    assert sorted(r.paths()) == ["a/b/c", "a/i32", "empty", "f32", "u"]
    np.testing.assert_array_equal(r.read("a/b/c"), np.arange(12.0).reshape(4, 3))
    assert r.read("a/i32", h5.I64)[0, 0] == -3            # converted on read
    np.testing.assert_array_equal(r.read("u", h5.F64), [1.0, 2.0, 3.0])
    assert r.read("empty", h5.I64).shape == (0,)
    np.testing.assert_array_equal(r.read("f32"), [1.5, -2.25])


def test_h5_many_groups(tmp_path):
    # a root group with hundreds of members (one P_%05u group per particle)
    w = h5.Writer()
    for p in range(600):
        w.add("P_%05d/x" % p, np.array([[p]], dtype=np.int64))
    f = tmp_path / "many.h5"
    w.write(f)
    r = h5.Reader(f)
    assert len(r.paths()) == 600
    assert r.read("P_00599/x", h5.I64)[0, 0] == 599


def test_h5_rejects_non_hdf5(tmp_path):
    f = tmp_path / "bad.h5"
    f.write_bytes(b"not an hdf5 file at all" * 10)
    with pytest.raises(OSError):
        h5.Reader(f)


def test_estimate_bytes_runs_on_the_host_and_checks_indices():
    """pd_estimate_bytes is host work only (admission control calls it before any device
    work): it sizes both forms, grows with the batch, and refuses a Connectivity index out of
    range as pd_create_batch does."""
    L = _capi.lib()
    s, _ = cases.impact_walls(steps=10)
    st, keep = _capi.setup_struct(s)
    pair = (_capi.PdSetupArrays * 2)(st, st)
    b1, b2 = C.c_uint64(), C.c_uint64()
    for prec in (0, 1):
        assert L.pd_estimate_bytes(C.byref(st), 1, prec, C.byref(b1)) == 0
        assert L.pd_estimate_bytes(pair, 2, prec, C.byref(b2)) == 0
        assert 0 < b1.value < b2.value
    s.conn = s.conn.copy()
    s.conn[5, 1] = s.n_nodes + 7
    bad, keep2 = _capi.setup_struct(s)
    assert L.pd_estimate_bytes(C.byref(bad), 1, 1, C.byref(b1)) == _capi.PD_EINVAL
    assert b"out of range" in L.pd_global_error()
