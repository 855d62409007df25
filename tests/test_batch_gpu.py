"""Batches of independent simulations and the serving loop, through the C-ABI batch entry
points (pd_create_batch, pd_finish_sim, pd_get_sim_state, pd_get_sim_damage, ...).

A simulation inside a batch must compute exactly what it computes alone: every quantity is
compared bit for bit with a handle of its own, in both precision forms. The serving loop
must return, for every request, that same result whatever else was resident meanwhile."""
import numpy as np
import pytest

from peridem_gb300 import serve
from peridem_gb300.sim import Batch, Sim, estimate_bytes
from tests import cases

pytestmark = pytest.mark.gpu

MIX = ["impact_walls", "cubes_gravity", "toggles", "impact_free"]


def _alone(name, precision, steps):
    s, cfg = cases.CASES[name]()
    sim = Sim(s, cfg, precision)
    sim.step(steps)
    out = sim.state(), sim.wall(), [sim.connectivity(p) for p in range(s.n_particles)], sim.damage()
    sim.close()
    return out


def _check_same(b, i, ref, name):
    st, (w, r), conn, dmg = ref
    a = b.sim_state(i)
    for k in ("curpos", "vel", "acc", "force", "disp"):
        np.testing.assert_array_equal(a[k], st[k], err_msg=f"{name} {k}")
    wb, rb = b.sim_wall(i)
    np.testing.assert_array_equal(wb, w)
    np.testing.assert_array_equal(rb, r)
    for p, c in enumerate(conn):
        np.testing.assert_array_equal(b.sim_connectivity(i, p), c, err_msg=f"{name} conn {p}")
    np.testing.assert_array_equal(b.sim_damage(i), dmg, err_msg=f"{name} damage")


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_batch_member_equals_alone(precision):
    items = [cases.CASES[n]() for n in MIX]
    b = Batch([s for s, _ in items], [c for _, c in items], precision)
    assert b.n_sims == len(MIX)
    b.step(25)
    for i, n in enumerate(MIX):
        _check_same(b, i, _alone(n, precision, 25), n)
        assert b.sim_steps(i) == 25
    b.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_finished_member_keeps_its_state(precision):
    names = ["impact_walls", "cubes_gravity"]
    items = [cases.CASES[n]() for n in names]
    b = Batch([s for s, _ in items], [c for _, c in items], precision)
    b.step(10)
    b.finish(0)
    b.step(15)
    assert b.sim_steps(0) == 10 and b.sim_steps(1) == 25
    _check_same(b, 0, _alone(names[0], precision, 10), names[0])
    _check_same(b, 1, _alone(names[1], precision, 25), names[1])
    b.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_estimate_equals_device_bytes(precision):
    items = [cases.CASES[n]() for n in MIX]
    setups = [s for s, _ in items]
    est = estimate_bytes(setups, precision)
    b = Batch(setups, [c for _, c in items], precision)
    assert est == b.device_bytes()
    b.close()


def test_server_results_equal_alone():
    # request 1 runs long enough that the later arrivals are admitted as other cohorts while
    # it is still resident: results must not depend on what runs beside them
    names = ["impact_walls", "cubes_gravity", "impact_free", "toggles", "impact_walls"]
    steps = [30, 3000, 20, 28, 12]
    arrivals = [0.0, 0.0, 0.05, 0.15, 0.3]
    reqs = []
    for rid, (n, k, t) in enumerate(zip(names, steps, arrivals)):
        s, cfg = cases.CASES[n]()
        reqs.append(serve.Request(rid, s, cfg, k, t))
    srv = serve.Server("fp32c", chunk_steps=7, max_batch=3, keep_damage=True)
    res = srv.run(reqs)
    assert srv.used == 0 and not srv.cohorts
    for r, n, k in zip(res, names, steps):
        assert r.error is None and r.steps == k
        st, wall, _, dmg = _alone(n, "fp32c", k)
        np.testing.assert_array_equal(r.damage, dmg, err_msg=f"request {r.rid} damage")
        for key in ("curpos", "vel", "acc", "force"):
            np.testing.assert_array_equal(r.state[key], st[key], err_msg=f"request {r.rid} {key}")
        np.testing.assert_array_equal(r.wall[0], wall[0])
        assert r.done >= r.arrival
    summ = serve.summarize(res, max(r.done for r in res))
    assert summ["completed"] == len(reqs) and summ["ttc_p99_s"] >= summ["ttc_p50_s"] > 0
    assert srv.max_resident >= 2  # two cohorts were on the device at once


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_server_compaction_results_equal_alone(precision):
    """Budget for three requests: a long one shares the first cohort with two short ones while
    three more wait. When the short ones finish, the cohort is compacted -- the long request is
    saved to host memory, the handle closed, and the request continues in the next cohort with
    the waiting ones (possibly several times). Every result equals the simulation run alone, bit
    for bit."""
    names = ["impact_walls", "impact_free", "impact_walls", "impact_free", "impact_walls", "impact_free"]
    steps = [90, 12, 15, 20, 25, 18]
    reqs = []
    for rid, (n, k) in enumerate(zip(names, steps)):
        s, cfg = cases.CASES[n]()
        reqs.append(serve.Request(rid, s, cfg, k, 0.0))
    per = max(estimate_bytes([r.setup], precision) for r in reqs)
    srv = serve.Server(precision, capacity_bytes=3 * per, chunk_steps=5, max_batch=3, keep_damage=True)
    res = srv.run(reqs, realtime=False)
    assert srv.evictions >= 1 and [e for e in srv.log if e[1] == "evict"]
    assert srv.used == 0 and not srv.cohorts
    for r, n, k in zip(res, names, steps):
        assert r.error is None and r.steps == k
        st, wall, conn, dmg = _alone(n, precision, k)
        for key in ("curpos", "vel", "acc", "force"):
            np.testing.assert_array_equal(r.state[key], st[key], err_msg=f"request {r.rid} {key}")
        np.testing.assert_array_equal(r.wall[0], wall[0])
        np.testing.assert_array_equal(r.wall[1], wall[1])
        np.testing.assert_array_equal(r.damage, dmg, err_msg=f"request {r.rid} damage")
