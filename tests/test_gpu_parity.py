"""GPU parity against the CPU oracle, through the C-ABI (peridem_gb300.sim.Sim wraps
include/peridem_gb300.h).

FP64 form: bit-exact. Every saved quantity of the reference's frames (CurrPos, vel, acc,
force, Connectivity, wall position) must be identical; the wall reaction, which the GPU sums
with atomics in a different order, must agree to 1e-12 relative.
FP32-compensated form: displacements within 1e-5 of the largest displacement magnitude and
broken-bond sets within 0.1% of the FP64 oracle's."""
import numpy as np
import pytest

from oracle import oracle as O
from peridem_gb300._capi import lib
from peridem_gb300.sim import Sim
from tests import cases

pytestmark = pytest.mark.gpu


def _compare_exact(name, s, sim, orc, t):
    a = sim.state()
    b = orc.state()
    for k in ("curpos", "vel", "acc", "force", "disp"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=f"{name} t={t} {k}")
    for p in range(s.n_particles):
        np.testing.assert_array_equal(sim.connectivity(p), orc.connectivity(p), err_msg=f"{name} t={t} conn {p}")
    wg, rg = sim.wall()
    wo, ro = orc.wall()
    np.testing.assert_array_equal(wg, wo)
    scale = max(1e-300, np.abs(ro).max())
    assert np.abs(rg - ro).max() <= 1e-12 * scale, f"{name} reaction"
    np.testing.assert_array_equal(sim.aabb(), orc.aabb())
    np.testing.assert_array_equal(sim.applied_force_density(), orc.afd(), err_msg=f"{name} t={t} afd")


@pytest.mark.parametrize("name", sorted(cases.CASES))
def test_fp64_bitexact(name):
    s, cfg = cases.CASES[name]()
    steps = cfg["timesteps"]
    sim = Sim(s, cfg, "fp64")
    sim.tune(stats=1)
    orc = O.Oracle(s, cfg)
    chunk = max(1, steps // 3)
    t = 0
    while t < steps:
        k = min(chunk, steps - t)
        sim.step(k)
        orc.step(k)
        t += k
        _compare_exact(name, s, sim, orc, t)
        st = sim.stats()
        oc = orc.counts()
        assert st["live_bonds"] == oc["live_bonds"]
        assert st["contacts"] == oc["contacts"]
    sim.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
@pytest.mark.parametrize("mode", [0, 2, 3])
@pytest.mark.parametrize("name", ["impact_walls", "cubes_gravity"])
def test_launch_modes_give_the_same_results(name, mode, precision):
    """Separate launches (0), the step graph with the broad phase in a conditional node (2, the
    default on large handles) and the persistent step (3, the FP32 default on small handles; FP64
    handles fall back to 2) against the plain step graph (1), rebuilds included."""
    s, cfg = cases.CASES[name]()
    a = Sim(s, cfg, precision)
    b = Sim(s, cfg, precision)
    a.tune(graphs=1)
    b.tune(graphs=mode)
    a.step(25)
    b.step(25)
    if mode == 2 or (mode == 3 and precision == "fp64"):
        assert b.graph_mode() in (1, 2)  # 1 where the conditional node is unsupported
    if mode == 3 and precision == "fp32c":
        assert b.graph_mode() == 3
    sa, sb = a.state(), b.state()
    for k in sa:
        np.testing.assert_array_equal(sa[k], sb[k])
    assert a.stats()["rebuilds"] == b.stats()["rebuilds"] > 0


@pytest.mark.parametrize("skin", [0.05, 0.2, 1.0])
def test_fp64_skin_does_not_change_results(skin):
    s, cfg = cases.impact_free()
    a = Sim(s, cfg, "fp64")
    a.tune(skin_frac=skin)
    orc = O.Oracle(s, cfg)
    a.step(cfg["timesteps"])
    orc.step(cfg["timesteps"])
    np.testing.assert_array_equal(a.state()["curpos"], orc.state()["curpos"])


def test_two_sphere_full_size_bitexact():
    """Config 0 at full size (2 x 4169 nodes, 7.4e5 bonds), first 60 steps."""
    from peridem_gb300 import gen
    s, cfg = gen.two_sphere()
    sim = Sim(s, cfg, "fp64")
    orc = O.Oracle(s, cfg)
    sim.step(60)
    orc.step(60)
    a, b = sim.state(), orc.state()
    for k in ("curpos", "vel", "acc", "force"):
        np.testing.assert_array_equal(a[k], b[k])


@pytest.mark.parametrize("name", ["impact_free", "cubes_gravity", "impact_walls", "prescribed", "toggles",
                                  "bdry_only", "notched"])
def test_fp32c_within_tolerance(name):
    s, cfg = cases.CASES[name]()
    steps = cfg["timesteps"]
    sim = Sim(s, cfg, "fp32c")
    orc = O.Oracle(s, cfg)
    sim.step(steps)
    orc.step(steps)
    a, b = sim.state(), orc.state()
    dref = max(np.abs(b["disp"]).max(), 1e-300)
    err = np.abs(a["disp"] - b["disp"]).max() / dref
    assert err <= 1e-5, f"{name}: relative displacement error {err:.3e}"
    n_or = sum(len(orc.connectivity(p)) for p in range(s.n_particles))
    mism = 0
    for p in range(s.n_particles):
        ca = {tuple(r) for r in sim.connectivity(p)}
        cb = {tuple(r) for r in orc.connectivity(p)}
        mism += len(ca ^ cb)
    assert mism <= 1e-3 * max(1, n_or), f"{name}: {mism} bond mismatches of {n_or}"


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_snapshot_restore_replays_identically(precision):
    s, cfg = cases.impact_free()
    sim = Sim(s, cfg, precision)
    sim.step(10)
    sim.snapshot()
    sim.step(15)
    a = sim.state()
    ca = [sim.connectivity(p) for p in range(s.n_particles)]
    sim.restore()
    sim.step(15)
    b = sim.state()
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])
    for p in range(s.n_particles):
        np.testing.assert_array_equal(ca[p], sim.connectivity(p))


def test_autotune_is_result_neutral():
    s, cfg = cases.cubes_gravity()
    a = Sim(s, cfg, "fp32c")
    b = Sim(s, cfg, "fp32c")
    a.step(5)
    b.step(5)
    chosen, ms = a.autotune(4)
    assert 0 <= chosen < len(ms) and np.all(ms > 0)
    a.step(20)
    b.step(20)
    sa, sb = a.state(), b.state()
    for k in sa:
        np.testing.assert_array_equal(sa[k], sb[k])
    for v in range(len(ms)):
        c = Sim(s, cfg, "fp32c")
        c.set_variant(v)
        c.step(25)
        np.testing.assert_array_equal(c.state()["curpos"], sa["curpos"])


def test_fp32c_restore_after_breaking():
    """Bonds broken after a snapshot come back with the restore (the FP32 kernels keep a broken
    flag in each column entry besides the live masks) and the replay is identical."""
    s, cfg = cases.impact_free(steps=60)
    sim = Sim(s, cfg, "fp32c")
    sim.step(5)
    sim.snapshot()
    n0 = sim.live_bonds()
    sim.step(40)
    n1 = sim.live_bonds()
    assert n1 < n0, "the case must break bonds after the snapshot"
    a = sim.state()
    ca = [sim.connectivity(p) for p in range(s.n_particles)]
    sim.restore()
    assert sim.live_bonds() == n0
    sim.step(40)
    assert sim.live_bonds() == n1
    b = sim.state()
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])
    for p in range(s.n_particles):
        np.testing.assert_array_equal(ca[p], sim.connectivity(p))


def test_fp32c_variants_identical_with_breaking():
    """Every bond-kernel variant, and an autotune run in the middle of the fracture, gives the
    same state and the same broken bonds."""
    s, cfg = cases.impact_free(steps=60)
    ref = Sim(s, cfg, "fp32c")
    n0 = ref.live_bonds()
    ref.step(40)
    ra = ref.state()
    rc = [ref.connectivity(p) for p in range(s.n_particles)]
    assert ref.live_bonds() < n0, "the case must break bonds"
    t = Sim(s, cfg, "fp32c")
    t.step(20)
    t.autotune(3)
    t.step(20)
    tb = t.state()
    for k in ra:
        np.testing.assert_array_equal(ra[k], tb[k])
    for v in range(lib().pd_num_variants()):
        c = Sim(s, cfg, "fp32c")
        c.set_variant(v)
        c.step(40)
        np.testing.assert_array_equal(c.state()["curpos"], ra["curpos"], err_msg=f"variant {v}")
        for p in range(s.n_particles):
            np.testing.assert_array_equal(c.connectivity(p), rc[p], err_msg=f"variant {v} conn {p}")


def test_fp64_bitexact_with_unsorted_connectivity():
    """A Connectivity in arbitrary order (pairs shuffled, some written (j, i)): rows keep the
    reference's push order, so the FP64 form still matches the oracle bit for bit (the device
    bond build covers sorted files; this one takes the host build)."""
    s, cfg = cases.impact_walls(steps=20)
    rng = np.random.default_rng(5)
    conn = s.conn.copy()
    for p in range(s.n_particles):
        a, b = int(s.conn_offset[p]), int(s.conn_offset[p + 1])
        blk = conn[a:b][rng.permutation(b - a)]
        flip = rng.random(b - a) < 0.5
        blk[flip] = blk[flip][:, ::-1]
        conn[a:b] = blk
    s.conn = np.ascontiguousarray(conn)
    sim = Sim(s, cfg, "fp64")
    orc = O.Oracle(s, cfg)
    sim.step(20)
    orc.step(20)
    _compare_exact("unsorted", s, sim, orc, 20)


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_damage_field(precision):
    """pd_get_damage (computed on the device) equals the plotting script's damage of the
    Connectivity the handle returns, bit for bit; in the FP64 form that Connectivity is the
    oracle's. Node 0 of particle 0 has every setup pair removed, so its damage is NaN (0/0)."""
    s, cfg = cases.impact_walls(steps=40)
    a, b = int(s.conn_offset[0]), int(s.conn_offset[1])
    keep = np.ones(len(s.conn), dtype=bool)
    keep[a:b] = (s.conn[a:b] != 0).all(axis=1)
    s.conn = np.ascontiguousarray(s.conn[keep])
    s.conn_offset = s.conn_offset - np.concatenate([[0], np.full(s.n_particles, b - a - keep[a:b].sum())]).astype(
        s.conn_offset.dtype)
    sim = Sim(s, cfg, precision)
    d0 = sim.damage()
    assert np.isnan(d0[0]) and np.isnan(d0).sum() == 1
    np.testing.assert_array_equal(d0[1:], 0.0)
    sim.step(40)
    d = sim.damage()
    conns = [sim.connectivity(p) for p in range(s.n_particles)]
    np.testing.assert_array_equal(d, O.damage(s, conns))
    assert np.nanmax(d) > 0, "the case must break bonds"
    if precision == "fp64":
        orc = O.Oracle(s, cfg)
        orc.step(40)
        np.testing.assert_array_equal(d, O.damage(s, [orc.connectivity(p) for p in range(s.n_particles)]))
