"""Checks against golden frames written by PeriDEM's own code (tests/golden/make_golden.py):
the CPU oracle everywhere (it must reproduce the reference bit for bit), and the GPU FP64 form
through the C-ABI on a GPU."""
import numpy as np
import pytest

from tests.golden.make_golden import load
from oracle import oracle as O
from tests import cases

NAMES = sorted(cases.CASES)


def _check(name, g, t, counter, curpos, vel, acc, force, conn_fn, wall, reaction, afd=None):
    f = g["frames"][counter]
    for p, ref in f.get("afd", {}).items():
        sl = g["setup"].particle_slice(p)
        np.testing.assert_array_equal(afd[sl], ref, err_msg=f"{name} frame {counter} applied_force_density")
    np.testing.assert_array_equal(curpos, f["CurrPos"], err_msg=f"{name} frame {counter} CurrPos")
    np.testing.assert_array_equal(vel, f["vel"], err_msg=f"{name} frame {counter} vel")
    np.testing.assert_array_equal(acc, f["acc"], err_msg=f"{name} frame {counter} acc")
    np.testing.assert_array_equal(force, f["force"], err_msg=f"{name} frame {counter} force")
    s = g["setup"]
    co = f["conn_offset"]
    for p in range(s.n_particles):
        np.testing.assert_array_equal(conn_fn(p).astype(np.int64), f["conn"][co[p]:co[p + 1]])
    np.testing.assert_array_equal(wall, f["wall_info"])
    if "reaction" in f and reaction is not None:
        scale = max(1e-300, np.abs(f["reaction"]).max())
        assert np.abs(reaction - f["reaction"]).max() <= 1e-12 * scale


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_golden(name):
    from oracle import oracle as O
    g = load(name)
    cfg = g["config"]
    orc = O.Oracle(g["setup"], cfg)
    t = 0
    for counter in sorted(g["frames"]):
        orc.step(cfg["modulo"])
        t += cfg["modulo"]
        st = orc.state()
        w, r = orc.wall()
        _check(name, g, t, counter, st["curpos"], st["vel"], st["acc"], st["force"], orc.connectivity, w, r,
               orc.afd())


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_fp64_matches_reference_golden(name):
    from peridem_gb300.sim import Sim
    g = load(name)
    cfg = g["config"]
    sim = Sim(g["setup"], cfg, "fp64")
    t = 0
    for counter in sorted(g["frames"]):
        sim.step(cfg["modulo"])
        t += cfg["modulo"]
        st = sim.state()
        w, r = sim.wall()
        _check(name, g, t, counter, st["curpos"], st["vel"], st["acc"], st["force"], sim.connectivity, w, r,
               sim.applied_force_density())
    sim.close()


def test_oracle_cell_search_equals_brute_force():
    """The oracle's cell-search contact (used to check large cases) gives the brute-force loops'
    results bit for bit on every small case, contacts and self-contact included."""
    from tests import cases
    for name in sorted(cases.CASES):
        s, cfg = cases.CASES[name]()
        a = O.Oracle(s, cfg)
        b = O.Oracle(s, cfg, cell_search=True)
        for _ in range(3):
            k = max(1, cfg["timesteps"] // 3)
            a.step(k)
            b.step(k)
            sa, sb = a.state(), b.state()
            for key in sa:
                np.testing.assert_array_equal(sa[key], sb[key], err_msg=f"{name} {key}")
            assert a.counts() == b.counts(), name
            for p in range(s.n_particles):
                np.testing.assert_array_equal(a.connectivity(p), b.connectivity(p))
            np.testing.assert_array_equal(a.wall()[1], b.wall()[1])


def test_oracle_cell_search_equals_brute_force_on_a_packing_in_contact():
    """Eight overlapping particles pressed by the top wall (inter-particle and self-contact,
    breaking): 10 steps by both contact loops, bit for bit."""
    from peridem_gb300 import gen
    MM = 1e-3
    s, cfg = gen.crush512(n=2, box=2.2 * MM, steps=10, dt=5e-9, hs=(0.075 * MM, 0.1 * MM), smin=1.2 * MM,
                          smax=1.4 * MM)
    cfg.update(wall_z_max=float(s.pos[:, 2].max()) + 0.02 * MM, speed_wall_z_max=-20.0, compute_wall_reaction=1)
    a = O.Oracle(s, cfg)
    b = O.Oracle(s, cfg, cell_search=True)
    a.step(10)
    b.step(10)
    sa, sb = a.state(), b.state()
    for key in sa:
        np.testing.assert_array_equal(sa[key], sb[key], err_msg=key)
    assert a.counts() == b.counts()
    broken = len(s.conn) - sum(len(a.connectivity(p)) for p in range(s.n_particles))
    assert broken > 0
    for p in range(s.n_particles):
        np.testing.assert_array_equal(a.connectivity(p), b.connectivity(p))
