"""Pins the CPU oracle to PeriDEM's own code: the reference's run/simulate3d.cpp and src/*.h
compiled against stand-in Eigen/MPI/HDF5 headers (oracle/_ref), run through its own main()
on the same setup and main.conf. Every saved frame must agree bit for bit. Runs where the
reference sources exist (they are not shipped to GPU machines); elsewhere the committed
golden fixtures (test_golden.py) carry the same check."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import cases

pytestmark = pytest.mark.skipif(not O.ref_available(), reason="reference not built on this machine")


@pytest.mark.parametrize("name", sorted(cases.CASES))
def test_oracle_matches_reference(name):
    s, cfg = cases.CASES[name]()
    steps = cfg["timesteps"]
    cfg = dict(cfg, save_file=1, modulo=max(1, steps // 3))
    frames = O.run_reference(s, cfg)
    orc = O.Oracle(s, cfg)
    counters = sorted(k for k in frames if isinstance(k, int))
    assert counters, "reference wrote no frames"
    t = 0
    for cnt in counters:
        orc.step(cfg["modulo"])
        t += cfg["modulo"]
        st = orc.state()
        ref = frames[cnt]["particles"]
        for p in range(s.n_particles):
            sl = s.particle_slice(p)
            for kr, ko in (("CurrPos", "curpos"), ("vel", "vel"), ("acc", "acc"), ("force", "force")):
                np.testing.assert_array_equal(ref[p][kr], st[ko][sl], err_msg=f"{name} t={t} p={p} {kr}")
            np.testing.assert_array_equal(ref[p]["Connectivity"], orc.connectivity(p).astype(np.int64))
            if "applied_force_density" in ref[p]:
                np.testing.assert_array_equal(ref[p]["applied_force_density"], orc.afd()[sl],
                                              err_msg=f"{name} t={t} p={p} applied_force_density")
        w, r = orc.wall()
        np.testing.assert_array_equal(frames[cnt]["wall"]["wall_info"].ravel(), w)
        if frames[cnt]["wall"]["reaction"] is not None:
            np.testing.assert_array_equal(frames[cnt]["wall"]["reaction"], r)
    pi = frames["plotinfo"]
    assert int(pi["dimension"].ravel()[0]) == 3
    assert float(pi["dt"].ravel()[0]) == cfg["dt"]
