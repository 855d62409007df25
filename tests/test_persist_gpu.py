"""The persistent step (launch mode 3): all steps of a pd_step call in one cooperative launch of
the FP32 form, its phases separated by grid barriers, against the plain step graph (mode 1).

The persistent kernel calls the same device code as the step graph's kernels, so every quantity
must agree bit for bit: positions, velocities, accelerations, forces, displacements, walls and
their reactions, the surviving bonds, the rebuild count. The cases cover contact rebuilds,
walls, fracture, scheduled toggles with clamped nodes, batches with members that finish early,
odd step counts (the state's double buffer changes parity inside a launch) and calls cut at the
per-launch step limit."""
import numpy as np
import pytest

from peridem_gb300.sim import Batch, Sim
from tests import cases

pytestmark = pytest.mark.gpu


def _no_torque_toggles(steps=30):
    """toggles() without the torque schedule (torque particles keep a handle off mode 3)."""
    s, cfg = cases.toggles(steps)
    s.torque_val[:] = 0.0
    cfg.update(set_torque_timestep=-1, enable_torque=0)
    return s, cfg


PCASES = {
    "impact_walls": cases.impact_walls,
    "impact_free": cases.impact_free,
    "cubes_gravity": cases.cubes_gravity,
    "notched": cases.notched,
    "toggles_clamped": _no_torque_toggles,
}


def _compare(a, b, n_particles, tag):
    sa, sb = a.state(), b.state()
    for k in sa:
        np.testing.assert_array_equal(sa[k], sb[k], err_msg=f"{tag} {k}")
    wa, ra = a.wall()
    wb, rb = b.wall()
    np.testing.assert_array_equal(wa, wb, err_msg=f"{tag} wall")
    np.testing.assert_array_equal(ra, rb, err_msg=f"{tag} reaction")
    for p in range(n_particles):
        np.testing.assert_array_equal(a.connectivity(p), b.connectivity(p), err_msg=f"{tag} conn {p}")


@pytest.mark.parametrize("lanes", [0, 1, 2, 4])
@pytest.mark.parametrize("chunks", [(25,), (7, 1, 17)])
@pytest.mark.parametrize("name", sorted(PCASES))
def test_persistent_step_equals_step_graph(name, chunks, lanes):
    s, cfg = PCASES[name]()
    a = Sim(s, cfg, "fp32c")
    b = Sim(s, cfg, "fp32c")
    a.tune(graphs=1)
    b.tune(graphs=3)
    b.set_persist_lanes(lanes)
    assert b.graph_mode() == 3
    for n in chunks:
        a.step(n)
        b.step(n)
    _compare(a, b, s.n_particles, name)
    sa, sb = a.stats(), b.stats()
    assert sa["rebuilds"] == sb["rebuilds"] > 0
    assert sa["step"] == sb["step"]
    assert sb["device_errors"] == 0
    a.close()
    b.close()


@pytest.mark.parametrize("lanes", [0, 4])
def test_lanes_on_a_mid_size_aggregate(lanes):
    """53k nodes, more than one resident thread each for four lanes per node: lanes 0 takes one
    lane per node (the gather-ahead loop), lanes 4 has each warp loop over several 8-node slices;
    both bit-identical to the step graph."""
    from peridem_gb300 import gen
    s, cfg = gen.aggregate(20, seed=7, steps=100)
    a = Sim(s, cfg, "fp32c")
    b = Sim(s, cfg, "fp32c")
    a.tune(graphs=1)
    b.tune(graphs=3)
    b.set_persist_lanes(lanes)
    a.step(30)
    b.step(30)
    _compare(a, b, s.n_particles, "aggregate 53k")
    a.close()
    b.close()


def test_persistent_step_beyond_one_launch():
    """More steps than one persistent launch takes (1024): the call is cut into launches."""
    s, cfg = cases.impact_free(steps=1100)
    a = Sim(s, cfg, "fp32c")
    b = Sim(s, cfg, "fp32c")
    a.tune(graphs=1)
    b.tune(graphs=3)
    a.step(1100)
    b.step(1100)
    _compare(a, b, s.n_particles, "1100 steps")
    a.close()
    b.close()


def test_persistent_step_with_overflowing_candidate_lists():
    """Lists of 2 candidates overflow in contact: those nodes walk the cell list, in both modes,
    and the lists grow at the same pd_step calls."""
    s, cfg = cases.impact_walls()
    a = Sim(s, cfg, "fp32c")
    b = Sim(s, cfg, "fp32c")
    a.tune(graphs=1, cand_cap=2)
    b.tune(graphs=3, cand_cap=2)
    for n in (10, 10, 10):
        a.step(n)
        b.step(n)
    _compare(a, b, s.n_particles, "cand_cap 2")
    a.close()
    b.close()


def test_persistent_batch_with_finished_member():
    names = ["impact_walls", "cubes_gravity", "impact_free"]
    items = [cases.CASES[n]() for n in names]
    ba = Batch([s for s, _ in items], [c for _, c in items], "fp32c")
    bb = Batch([s for s, _ in items], [c for _, c in items], "fp32c")
    ba.tune(graphs=1)
    bb.tune(graphs=3)
    assert bb.graph_mode() == 3
    for b in (ba, bb):
        b.step(9)
        b.finish(1)
        b.step(14)
    for i in range(len(names)):
        sa, sb = ba.sim_state(i), bb.sim_state(i)
        for k in sa:
            np.testing.assert_array_equal(sa[k], sb[k], err_msg=f"{names[i]} {k}")
        np.testing.assert_array_equal(ba.sim_wall(i)[1], bb.sim_wall(i)[1])
        assert ba.sim_steps(i) == bb.sim_steps(i)
    ba.close()
    bb.close()


def test_persist_lanes_out_of_range_is_rejected():
    from peridem_gb300.sim import PdError
    s, cfg = cases.impact_free()
    a = Sim(s, cfg, "fp32c")
    with pytest.raises(PdError):
        a.set_persist_lanes(3)
    a.set_persist_lanes(2)
    assert a.persist_lanes() == 2
    a.close()


@pytest.mark.parametrize("precision,stats", [("fp64", -1), ("fp32c", 1)])
def test_persistent_mode_falls_back_where_not_eligible(precision, stats):
    """FP64 handles and handles with statistics on step with the conditional step graph."""
    s, cfg = cases.impact_walls()
    a = Sim(s, cfg, precision)
    a.tune(graphs=3, stats=stats)
    a.step(3)
    assert a.graph_mode() in (1, 2)
    a.close()


@pytest.mark.parametrize("workload", ["two_sphere", "cubes125"])
def test_small_benchmark_configurations_equal_step_graph(workload):
    """The two small benchmark configurations at full size (8,338 and 64,000 nodes): the default
    launch (the persistent step) and the autotuned one equal the plain step graph bit for bit."""
    from peridem_gb300 import gen
    s, cfg = getattr(gen, workload)()
    a = Sim(s, cfg, "fp32c")
    b = Sim(s, cfg, "fp32c")
    c = Sim(s, cfg, "fp32c")
    a.tune(graphs=1)
    c.autotune(2)
    for x in (a, b, c):
        x.step(40)
    assert b.graph_mode() == 3
    _compare(a, b, s.n_particles, workload + " default")
    _compare(a, c, s.n_particles, workload + " autotuned")
    for x in (a, b, c):
        x.close()


def test_autotune_with_rebuilds_keeps_results():
    """Two small spheres colliding in a wall box rebuild their candidate lists every few steps, so
    the autotuner also times wider contact skins; whatever it keeps, the results equal the untuned
    step graph's."""
    s, cfg = cases.impact_walls()
    a = Sim(s, cfg, "fp32c")
    b = Sim(s, cfg, "fp32c")
    b.autotune(2)
    a.tune(graphs=1)
    a.step(25)
    b.step(25)
    _compare(a, b, s.n_particles, "autotuned with rebuilds")
    assert b.stats()["rebuilds"] > 0
    a.close()
    b.close()


def test_autotune_may_pick_the_persistent_step():
    s, cfg = cases.cubes_gravity()
    a = Sim(s, cfg, "fp32c")
    b = Sim(s, cfg, "fp32c")
    b.autotune(4)
    assert b.graph_mode() in (1, 2, 3)
    a.tune(graphs=1)
    a.step(20)
    b.step(20)
    _compare(a, b, s.n_particles, "autotuned")
    a.close()
    b.close()
