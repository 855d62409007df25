"""Failure detection and recovery, with every failure made on the host (no GPU fault):

  * a NaN written into the displacement from the host makes the next force density
    non-finite: pd_sync reports PD_EDEVICE with the non-finite bit of the device error word
    (the reference would print and run on, src/debug/err.h:25-28), and the handle stays usable:
    the word clears, finite state can be written back and stepping resumes;
  * pd_sync(h, 0) only polls (PD_ETIMEOUT while steps are queued) and a bounded wait returns
    PD_ETIMEOUT when its limit passes first;
  * a contact-candidate list too short for a node (cand_cap 1 or 2) is not an error: that
    node's partners come from the cell list in the same order, so results equal the oracle's
    bit for bit (FP64) and the default capacity's bit for bit (FP32C), and the lists grow.
    The reference has no such capacity (contact.h:746-942 tests every node pair)."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from peridem_gb300 import _capi, gen
from peridem_gb300.sim import Sim
from tests import cases
from tests.test_gpu_parity import _compare_exact

pytestmark = pytest.mark.gpu
MM = 1e-3


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_nan_from_the_host_raises_the_non_finite_bit(precision):
    s, cfg = cases.impact_walls()
    sim = Sim(s, cfg, precision)
    sim.step(3)
    good = sim.state()
    bad = good["disp"].copy()
    bad[5, 1] = np.nan
    sim.set_state(disp=bad)
    sim.step(2, sync=False)
    rc = _capi.lib().pd_sync(sim.h, -1)
    assert rc == _capi.PD_EDEVICE
    msg = _capi.lib().pd_last_error(sim.h).decode()
    assert "non-finite" in msg, msg
    assert sim.stats()["device_errors"] & _capi.PD_DERR_NONFINITE
    # the handle is still usable: clear the word, write finite state, step on
    assert _capi.lib().pd_clear_device_errors(sim.h) == 0
    sim.set_state(disp=good["disp"], vel=good["vel"], acc=good["acc"])
    sim.step(2)
    assert sim.stats()["device_errors"] == 0
    assert np.isfinite(sim.state()["curpos"]).all()
    sim.close()


def test_sync_polls_and_bounded_waits_time_out():
    s, cfg = cases.cubes_gravity(steps=100000)
    sim = Sim(s, cfg, "fp32c")
    sim.step(2)
    sim.step(20000, sync=False)  # about a second of queued work
    L = _capi.lib()
    assert L.pd_sync(sim.h, 0) == _capi.PD_ETIMEOUT
    assert "queued" in L.pd_last_error(sim.h).decode()
    assert L.pd_sync(sim.h, 5) == _capi.PD_ETIMEOUT
    assert "timed out" in L.pd_last_error(sim.h).decode()
    assert L.pd_sync(sim.h, -1) == 0
    assert L.pd_sync(sim.h, 0) == 0
    sim.close()


def _packing(steps=12):
    s, cfg = gen.crush512(n=2, box=2.2 * MM, steps=steps, dt=5e-9, hs=(0.075 * MM, 0.1 * MM), smin=1.2 * MM,
                          smax=1.4 * MM)
    cfg.update(wall_z_max=float(s.pos[:, 2].max()) + 0.02 * MM, speed_wall_z_max=-20.0, compute_wall_reaction=1)
    return s, cfg


def _bytes(sim):
    b = C.c_uint64()
    assert _capi.lib().pd_device_bytes(sim.h, C.byref(b)) == 0
    return b.value


@pytest.mark.parametrize("name", ["impact_walls", "packing"])
def test_short_candidate_lists_give_the_oracle_results(name):
    s, cfg = _packing() if name == "packing" else cases.impact_walls()
    steps = cfg["timesteps"]
    sim = Sim(s, cfg, "fp64")
    sim.tune(cand_cap=1, stats=1)
    orc = O.Oracle(s, cfg)
    b0 = _bytes(sim)
    t = 0
    for k in (steps // 3, steps // 3, steps - 2 * (steps // 3)):
        sim.step(k)
        orc.step(k)
        t += k
        _compare_exact(name, s, sim, orc, t)
        assert sim.stats()["contacts"] == orc.counts()["contacts"]
        assert sim.stats()["device_errors"] == 0
    assert _bytes(sim) > b0  # the lists grew after the first chunk
    sim.close()


def test_short_candidate_lists_leave_fp32c_results_unchanged():
    s, cfg = _packing()
    a = Sim(s, cfg, "fp32c")
    b = Sim(s, cfg, "fp32c")
    b.tune(cand_cap=2)
    for _ in range(3):
        a.step(4)
        b.step(4)
    sa, sb = a.state(), b.state()
    for k in sa:
        np.testing.assert_array_equal(sa[k], sb[k], err_msg=k)
    for p in range(s.n_particles):
        np.testing.assert_array_equal(a.connectivity(p), b.connectivity(p))
    assert b.stats()["device_errors"] == 0
