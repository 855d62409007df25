"""The drop-in `simulate3d -c main.conf -i setup.h5 -o outdir` (run/simulate3d.cpp) end to end:
setup file in the reference's schema, main.conf in its grammar, frames out in its layout
(staged in stream order and written by a host thread while the steps go on).
Frames must equal the golden frames PeriDEM's own code wrote for the same case (bit for bit
in the FP64 form), and a resumed run (do_resume, timeloop.h:262-312) must equal the oracle
resumed from the same frame."""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from peridem_gb300 import h5
from tests.golden.make_golden import load

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent
EXE = ROOT / "peridem_gb300" / "_lib" / "simulate3d"


def run_cli(tmp_path, setup, cfg, precision="fp64"):
    out = tmp_path / "out"
    out.mkdir(exist_ok=True)
    h5.write_setup(tmp_path / "setup.h5", setup)
    O.write_conf(str(tmp_path / "main.conf"), cfg)
    r = subprocess.run([str(EXE), "-c", str(tmp_path / "main.conf"), "-i", str(tmp_path / "setup.h5"),
                        "-o", str(out), "-p", precision], capture_output=True, text=True, cwd=tmp_path, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return out, r.stdout


@pytest.mark.parametrize("name", ["impact_walls", "toggles", "cubes_gravity", "prescribed"])
def test_cli_frames_equal_reference_golden(tmp_path, name):
    g = load(name)
    s, cfg = g["setup"], g["config"]
    out, log = run_cli(tmp_path, s, cfg)
    assert "ct[1:" in log and "duration(s)" in log
    for counter, f in g["frames"].items():
        fr = h5.read_frame(out, counter, s.n_particles)
        parts = fr["particles"]
        for key in ("CurrPos", "vel", "acc", "force"):
            np.testing.assert_array_equal(np.concatenate([p[key] for p in parts]), f[key], err_msg=f"{key} {counter}")
        for p, ref in f.get("afd", {}).items():
            np.testing.assert_array_equal(parts[p]["applied_force_density"], ref, err_msg=f"afd {counter}")
        co = f["conn_offset"]
        for p in range(s.n_particles):
            np.testing.assert_array_equal(parts[p]["Connectivity"].astype(np.int64), f["conn"][co[p]:co[p + 1]])
        np.testing.assert_array_equal(fr["wall"]["wall_info"], f["wall_info"])
        if "reaction" in f:
            scale = max(1e-300, np.abs(f["reaction"]).max())
            assert np.abs(fr["wall"]["reaction"] - f["reaction"]).max() <= 1e-12 * scale
    pi = h5.Reader(out / "plotinfo.h5")
    assert int(pi.read("dimension", h5.I64).ravel()[0]) == 3
    assert pi.read("dt").ravel()[0] == cfg["dt"]
    np.testing.assert_array_equal(pi.read("f_l_counter", h5.I64).ravel(), [1, cfg["timesteps"] // cfg["modulo"]])


def test_cli_resume_equals_oracle_resume(tmp_path):
    g = load("impact_walls")
    s, cfg = g["setup"], dict(g["config"])
    out, _ = run_cli(tmp_path, s, cfg)
    k = 2
    fr = h5.read_frame(out, k, s.n_particles)
    # resume from frame k for one more save interval
    rcfg = dict(cfg, do_resume=1, resume_ind=k, wall_resume=1, timesteps=cfg["modulo"])
    O.write_conf(str(tmp_path / "main.conf"), rcfg)
    r = subprocess.run([str(EXE), "-c", str(tmp_path / "main.conf"), "-i", str(tmp_path / "setup.h5"),
                        "-o", str(out)], capture_output=True, text=True, cwd=tmp_path, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Resuming from counter 3" in r.stdout
    resumed = h5.read_frame(out, k + 1, s.n_particles)
    # the oracle resumed the same way: disp = CurrPos - pos, vel, acc, Connectivity, and the
    # saved walls (given to the oracle as config wall positions)
    cur = np.concatenate([p["CurrPos"] for p in fr["particles"]])
    w = fr["wall"]["wall_info"]
    orc2cfg = dict(rcfg, wall_x_min=w[0], wall_y_min=w[1], wall_z_min=w[2], wall_x_max=w[3], wall_y_max=w[4],
                   wall_z_max=w[5])
    orc = O.Oracle(s, orc2cfg)
    orc.set_state(disp=cur - s.pos, vel=np.concatenate([p["vel"] for p in fr["particles"]]),
                  acc=np.concatenate([p["acc"] for p in fr["particles"]]))
    for p in range(s.n_particles):
        orc.set_connectivity(p, fr["particles"][p]["Connectivity"])
    orc.step(cfg["modulo"])
    st = orc.state()
    np.testing.assert_array_equal(np.concatenate([p["CurrPos"] for p in resumed["particles"]]), st["curpos"])
    np.testing.assert_array_equal(np.concatenate([p["vel"] for p in resumed["particles"]]), st["vel"])
    for p in range(s.n_particles):
        np.testing.assert_array_equal(resumed["particles"][p]["Connectivity"], orc.connectivity(p))


def test_cli_fp32c_resume_close_to_oracle_resume(tmp_path):
    """The FP32-compensated form resumed from a frame with broken bonds: the saved Connectivity
    sets the live bits and the FP32 kernels' broken flags, so the resumed run stays within the
    form's tolerance of the oracle resumed from the same frame."""
    g = load("impact_walls")
    s, cfg = g["setup"], dict(g["config"])
    out, _ = run_cli(tmp_path, s, cfg, precision="fp32c")
    k = 2
    fr = h5.read_frame(out, k, s.n_particles)
    assert sum(len(p["Connectivity"]) for p in fr["particles"]) < len(s.conn), "the frame must have broken bonds"
    rcfg = dict(cfg, do_resume=1, resume_ind=k, wall_resume=1, timesteps=cfg["modulo"])
    O.write_conf(str(tmp_path / "main.conf"), rcfg)
    r = subprocess.run([str(EXE), "-c", str(tmp_path / "main.conf"), "-i", str(tmp_path / "setup.h5"),
                        "-o", str(out), "-p", "fp32c"], capture_output=True, text=True, cwd=tmp_path, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    resumed = h5.read_frame(out, k + 1, s.n_particles)
    cur = np.concatenate([p["CurrPos"] for p in fr["particles"]])
    w = fr["wall"]["wall_info"]
    orc = O.Oracle(s, dict(rcfg, wall_x_min=w[0], wall_y_min=w[1], wall_z_min=w[2], wall_x_max=w[3],
                           wall_y_max=w[4], wall_z_max=w[5]))
    orc.set_state(disp=cur - s.pos, vel=np.concatenate([p["vel"] for p in fr["particles"]]),
                  acc=np.concatenate([p["acc"] for p in fr["particles"]]))
    for p in range(s.n_particles):
        orc.set_connectivity(p, fr["particles"][p]["Connectivity"])
    orc.step(cfg["modulo"])
    st = orc.state()
    got = np.concatenate([p["CurrPos"] for p in resumed["particles"]])
    assert np.abs(got - st["curpos"]).max() <= 1e-5 * max(np.abs(st["disp"]).max(), 1e-300)
    n_or = sum(len(orc.connectivity(p)) for p in range(s.n_particles))
    mism = sum(len({tuple(x) for x in resumed["particles"][p]["Connectivity"]} ^
                   {tuple(x) for x in orc.connectivity(p)}) for p in range(s.n_particles))
    assert mism <= 1e-3 * max(1, n_or)


def test_cli_fp32c_close_to_reference(tmp_path):
    g = load("cubes_gravity")
    s, cfg = g["setup"], g["config"]
    out, _ = run_cli(tmp_path, s, cfg, precision="fp32c")
    last = max(g["frames"])
    fr = h5.read_frame(out, last, s.n_particles)
    cur = np.concatenate([p["CurrPos"] for p in fr["particles"]])
    ref = g["frames"][last]["CurrPos"]
    disp_ref = ref - s.pos
    assert np.abs(cur - ref).max() <= 1e-5 * np.abs(disp_ref).max()


def test_staged_frames_equal_synchronous_frames(tmp_path):
    """pd_run's frames (staged copies, writer thread) equal pd_write_frame's (synchronous reads)."""
    from peridem_gb300 import _capi
    import ctypes as C
    g = load("toggles")
    s, cfg = g["setup"], dict(g["config"])
    out, _ = run_cli(tmp_path, s, cfg)
    L = _capi.lib()
    sync_dir = tmp_path / "sync"
    sync_dir.mkdir()
    h = C.c_void_p()
    assert L.pd_open(str(tmp_path / "main.conf").encode(), str(tmp_path / "setup.h5").encode(),
                     str(sync_dir).encode(), 0, C.byref(h)) == 0
    for counter in range(1, cfg["timesteps"] // cfg["modulo"] + 1):
        assert L.pd_step(h, cfg["modulo"]) == 0
        assert L.pd_write_frame(h, counter) == 0
        a = h5.read_frame(out, counter, s.n_particles)
        b = h5.read_frame(sync_dir, counter, s.n_particles)
        for pa, pb in zip(a["particles"], b["particles"]):
            for k in pa:
                np.testing.assert_array_equal(pa[k], pb[k])
        np.testing.assert_array_equal(a["wall"]["wall_info"], b["wall"]["wall_info"])
    L.pd_close(h)


def test_cli_missing_setup_fails_cleanly(tmp_path):
    (tmp_path / "out").mkdir()
    r = subprocess.run([str(EXE), "-c", "nope.conf", "-i", str(tmp_path / "missing.h5"), "-o", str(tmp_path / "out")],
                       capture_output=True, text=True, cwd=tmp_path, timeout=120)
    assert r.returncode == 1
    assert "cannot open" in r.stderr
