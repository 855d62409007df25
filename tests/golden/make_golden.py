"""Generates tests/golden/*.npz: PeriDEM's own outputs on small seeded cases.

Runs the reference's run/simulate3d.cpp main() (built from the reference sources against
stand-in Eigen/MPI/HDF5 headers, oracle/_ref) on each case of tests/cases.py with
save_file = 1 and stores, per saved frame, what the reference writes to tc_%05u.h5 and
wall_%05u.h5 (CurrPos, vel, acc, force, Connectivity per particle, applied_force_density of a
prescribed-velocity particle; wall_info, reaction), next
to the setup arrays and the main.conf values used, so that tests on machines without the
reference sources can check against the reference's own results.

Usage (on a machine with the reference sources):  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402
from tests import cases  # noqa: E402

SETUP_KEYS = ("node_offset", "pos", "vol", "disp", "vel", "acc", "extforce", "conn_offset", "conn", "delta",
              "rho", "cnot", "snot", "torque_val", "movable", "breakable", "stoppable", "torque_axis",
              "bdry_offset", "bdry", "clamped_offset", "clamped")


def make(name: str) -> Path:
    s, cfg = cases.CASES[name]()
    steps = cfg["timesteps"]
    cfg = dict(cfg, save_file=1, modulo=max(1, steps // 3))
    frames = O.run_reference(s, cfg)
    out = {f"setup_{k}": getattr(s, k) for k in SETUP_KEYS}
    out["setup_scalars"] = np.array([s.contact_radius, s.normal_stiffness, s.damping_ratio,
                                     s.friction_coefficient, float(s.allow_wall)])
    out["setup_geom_wall_info"] = np.asarray(s.geom_wall_info)
    out["config_json"] = np.frombuffer(json.dumps(cfg).encode(), dtype=np.uint8)
    counters = sorted(k for k in frames if isinstance(k, int))
    out["counters"] = np.array(counters)
    for c in counters:
        parts = frames[c]["particles"]
        for key in ("CurrPos", "vel", "acc", "force"):
            out[f"f{c}_{key}"] = np.concatenate([p[key] for p in parts], axis=0)
        for pi, p in enumerate(parts):  # written for the prescribed-velocity particle only
            if "applied_force_density" in p:
                out[f"f{c}_afd_p{pi}"] = p["applied_force_density"]
        conns = [np.asarray(p["Connectivity"], dtype=np.int64).reshape(-1, 2) for p in parts]
        out[f"f{c}_conn_offset"] = np.concatenate([[0], np.cumsum([len(x) for x in conns])]).astype(np.int64)
        out[f"f{c}_conn"] = np.concatenate(conns, axis=0) if conns else np.zeros((0, 2), np.int64)
        out[f"f{c}_wall_info"] = frames[c]["wall"]["wall_info"].reshape(-1)
        r = frames[c]["wall"]["reaction"]
        if r is not None:
            out[f"f{c}_reaction"] = r
    path = Path(__file__).resolve().parent / f"{name}.npz"
    np.savez_compressed(path, **out)
    return path


def load(name: str) -> dict:
    """Returns {"setup": Setup, "config": dict, "frames": {counter: {...}}}."""
    from peridem_gb300.setupdata import Setup
    z = np.load(Path(__file__).resolve().parent / f"{name}.npz")
    sc = z["setup_scalars"]
    s = Setup(**{k: z[f"setup_{k}"] for k in SETUP_KEYS}, contact_radius=float(sc[0]),
              normal_stiffness=float(sc[1]), damping_ratio=float(sc[2]), friction_coefficient=float(sc[3]),
              allow_wall=int(sc[4]), geom_wall_info=z["setup_geom_wall_info"])
    cfg = json.loads(bytes(z["config_json"]).decode())
    frames = {}
    for c in z["counters"]:
        c = int(c)
        f = {k: z[f"f{c}_{k}"] for k in ("CurrPos", "vel", "acc", "force", "conn_offset", "conn", "wall_info")}
        if f"f{c}_reaction" in z:
            f["reaction"] = z[f"f{c}_reaction"]
        f["afd"] = {int(k.rsplit("_p", 1)[1]): z[k] for k in z.files if k.startswith(f"f{c}_afd_p")}
        frames[c] = f
    return {"setup": s, "config": cfg, "frames": frames}


if __name__ == "__main__":
    if not O.ref_available():
        raise SystemExit("the reference build (oracle/_ref) is missing: make -C oracle ref")
    for name in sorted(cases.CASES):
        p = make(name)
        print(name, p.stat().st_size, "bytes")
