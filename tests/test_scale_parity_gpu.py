"""FP64 parity at the size and particle mix of the benchmark configurations (through the C-ABI):
the plain FP64 GPU form against the oracle, bit for bit, on

  * the headline packing's own particle mix: the first 16 particles of crush512_4m (spheres,
    cubes and ellipsoids with lattice spacings 0.03, 0.045 and 0.06 mm side by side; 121,601
    nodes, 1.1e7 directed bonds), packed on a 1.2 mm pitch so that neighbours touch, with the top
    wall started at the packing and moving down at 20 m/s: node-node contact across lattices,
    wall contact with reaction and breaking all happen within the 20 steps;
  * cubes125 at its full size (125 rotated cubes, 64,000 nodes, 4.4e6 directed bonds) under
    gravity in its wall box;
  * a strip of the notched plate at h = 0.5 mm (60 x 40 x 9 mm, two 20 mm edge notches,
    181,415 nodes, 1.7e7 directed bonds) with the unbreakable impactor already in contact at
    200 m/s, so that contact and crack-tip breaking start at once.

The oracle visits only node pairs within reach in the reference's order (or_set_cell_search:
the same sums as the reference's brute-force loops, tested equal on every small case), so each
case checks in seconds. Every field the reference saves is compared bit for bit at three points
of the run, together with the live-bond and contact counts."""
import numpy as np
import pytest

from oracle import oracle as O
from peridem_gb300 import gen
from peridem_gb300.sim import Sim
from tests.test_gpu_parity import _compare_exact

pytestmark = pytest.mark.gpu
MM = 1e-3


def crush_contact(steps=20):
    return gen.crush_contact(steps=steps)


def cubes_full(steps=20):
    s, cfg = gen.cubes125(steps=steps)
    cfg.update(compute_wall_reaction=1)
    return s, cfg


def notched_strip(steps=20):
    return gen.notched_plate(Lx=60 * MM, Ly=40 * MM, notch_len=20 * MM, notch_x=(15 * MM, 45 * MM), imp_w=30 * MM,
                             imp_len=6 * MM, gap=-0.45, v=200.0, steps=steps)


def _run(name, s, cfg, steps=20, checkpoints=(7, 14, 20)):
    sim = Sim(s, cfg, "fp64")
    sim.tune(stats=1)
    orc = O.Oracle(s, cfg, cell_search=True)
    t = 0
    seen_contacts = 0
    for cp in checkpoints:
        sim.step(cp - t)
        orc.step(cp - t)
        t = cp
        _compare_exact(name, s, sim, orc, t)
        st, oc = sim.stats(), orc.counts()
        assert st["live_bonds"] == oc["live_bonds"], (name, t)
        assert st["contacts"] == oc["contacts"], (name, t)
        seen_contacts = max(seen_contacts, oc["contacts"])
    live = sum(len(orc.connectivity(p)) for p in range(s.n_particles))
    sim.close()
    return seen_contacts, len(s.conn) - live


def test_crush_mix_with_contact_walls_and_breaking():
    s, cfg = crush_contact()
    contacts, broken = _run("crush_contact", s, cfg)
    assert contacts > 0 and broken > 0


def test_cubes125_full_size():
    s, cfg = cubes_full()
    _run("cubes125", s, cfg)


def test_notched_plate_strip_in_contact():
    s, cfg = notched_strip()
    contacts, broken = _run("notched_strip", s, cfg)
    assert contacts > 0 and broken > 0
