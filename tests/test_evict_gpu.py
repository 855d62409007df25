"""Eviction and re-admission of a simulation (pd_save_sim / pd_load_sim, through the C-ABI).

A simulation is stepped in one batch, saved to host memory at a step boundary, its batch closed,
and loaded into a slot of a new batch with another companion simulation; stepped on, it must
equal the same simulation run alone from the start, bit for bit in both forms: every array the
reference saves in a frame, its Connectivity and the walls (the wall reaction, an output summed
with device atomics, to 1e-12 relative as in the other parity tests). The cases cover contact,
walls, breaking and self-contact (impact_walls), scheduled toggles with clamped nodes, torque
and gradient extforce (toggles), and a prescribed-velocity particle with reset_partzero_y
(prescribed): the checkpoint carries their state (afd, moved reference positions)."""
import numpy as np
import pytest

from peridem_gb300 import _capi
from peridem_gb300.sim import Batch, Sim
from tests import cases

pytestmark = pytest.mark.gpu


def _equal(a_state, b_state, what):
    for k in ("curpos", "vel", "acc", "force", "disp"):
        np.testing.assert_array_equal(a_state[k], b_state[k], err_msg=f"{what} {k}")


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
@pytest.mark.parametrize("name", ["impact_walls", "toggles", "prescribed"])
def test_evicted_and_readmitted_simulation_equals_alone(name, precision):
    s, cfg = cases.CASES[name]()
    other, ocfg = cases.cubes_gravity()
    steps = cfg["timesteps"]
    half = steps // 2
    alone = Sim(s, cfg, precision)
    alone.step(steps)
    # first half in a batch behind another simulation, then evicted
    b1 = Batch([other, s], [ocfg, cfg], precision)
    b1.step(half)
    blob = b1.save_sim(1)
    b1.close()
    # re-admitted into a new batch, in front of a fresh companion
    b2 = Batch([s, other], [cfg, ocfg], precision)
    b2.load_sim(blob, 0)
    assert b2.sim_steps(0) == half
    b2.step(steps - half)
    _equal(b2.sim_state(0), alone.state(), f"{name} {precision}")
    for p in range(s.n_particles):
        np.testing.assert_array_equal(b2.sim_connectivity(0, p), alone.connectivity(p))
    w2, r2 = b2.sim_wall(0)
    w1, r1 = alone.wall()
    np.testing.assert_array_equal(w2, w1)
    # the wall reaction is an output summed with device atomics (order-dependent rounding)
    assert np.abs(r2 - r1).max() <= 1e-12 * max(1e-300, np.abs(r1).max())
    # the companion is unaffected by the load: equal to a fresh run of its own
    comp = Sim(other, ocfg, precision)
    comp.step(steps - half)
    _equal(b2.sim_state(1), comp.state(), f"companion {precision}")
    for x in (alone, b2, comp):
        x.close()


def test_checkpoint_of_another_setup_is_refused():
    s, cfg = cases.impact_walls()
    o, ocfg = cases.cubes_gravity()
    a = Sim(s, cfg, "fp64")
    a.step(3)
    blob = a.save_sim(0)
    b = Sim(o, ocfg, "fp64")
    with pytest.raises(_capi.PdError) as e:
        b.load_sim(blob, 0)
    assert e.value.rc == _capi.PD_EINVAL
    c = Sim(s, cfg, "fp32c")  # same setup, other precision form
    with pytest.raises(_capi.PdError):
        c.load_sim(blob, 0)
    with pytest.raises(_capi.PdError):
        b.load_sim(blob[: len(blob) // 2], 0)
    for x in (a, b, c):
        x.close()


def test_a_finished_simulation_cannot_be_saved():
    s, cfg = cases.impact_walls()
    b = Batch([s, s], [cfg, cfg], "fp64")
    b.step(2)
    b.finish(0)
    with pytest.raises(_capi.PdError) as e:
        b.save_sim(0)
    assert e.value.rc == _capi.PD_ESTATE
    assert len(b.save_sim(1)) > 0
    b.close()
