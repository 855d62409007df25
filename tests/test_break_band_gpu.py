"""The FP32-compensated form's breaking decision far from a particle's anchor.

Its records hold positions and displacements as floats relative to an anchor node, so a bond
200 mm from the anchor carries rounding of ~1e-8 m on bond lengths of 0.5 mm, and a large rigid
rotation makes the displacements as large as the particle. The engine bounds the resulting
stretch error per particle and step (set_break_band: extent, shortest bond, rotation-proof
first-order bound) and re-takes every decision inside that band in FP64. Here a 200 x 3 x 3
mm steel bar at h = 0.5 mm, at rest or rigidly rotated by 0.6 or 1.3 rad, has bonds 70-100 mm
from its centre planted at stretches snot (1 + d), d from -0.2 to +0.2 (down to |d| = 3e-5,
four bonds per d); after one step
(zero velocity and acceleration, so the planted stretches are the ones evaluated) both forms
must break exactly the bonds with d > 0 (particle2.h:196-237: s > snot breaks)."""
import numpy as np
import pytest

from peridem_gb300 import gen
from peridem_gb300.sim import Sim

pytestmark = pytest.mark.gpu
MM = 1e-3
DELTAS = (3e-5, -3e-5, 6e-5, -6e-5, 1.2e-4, -1.2e-4, 2e-4, -2e-4, 1e-3, -1e-3, 5e-2, -5e-2, 0.2, -0.2)


def _rot(theta):
    c, s = np.cos(theta), np.sin(theta)
    rz = np.array([[c, -s, 0], [s, c, 0], [0, 0, 1.0]])
    c2, s2 = np.cos(0.5 * theta), np.sin(0.5 * theta)
    rx = np.array([[1.0, 0, 0], [0, c2, -s2], [0, s2, c2]])
    return rx @ rz


def bar_with_planted_bonds(theta):
    h = 0.5 * MM
    rng = np.random.default_rng(11)
    loc = gen.lattice("box", (200 * MM, 3.0 * MM, 3.0 * MM), h)
    part = gen.make_particle(loc, h, gen.STEEL, 3.0, rng, 0.05, (0.0, 0.0, 0.0))
    s = gen.finish([part], 0.5 * h, 1e-9)
    pos, conn = s.pos, s.conn.astype(np.int64)
    snot = float(s.snot[0])
    R = _rot(theta)
    disp = pos @ R.T - pos  # rigid rotation about the bar's centre
    # planted pairs: bonds nearly along the bar, more than 50 mm from its centre (the anchor),
    # farthest first, no two planted nodes bonded to each other
    xi = pos[conn[:, 1]] - pos[conn[:, 0]]
    ln = np.linalg.norm(xi, axis=1)
    axial = (np.abs(xi[:, 0]) > 0.9 * ln) & (ln < 1.5 * h) & (np.abs(pos[conn[:, 0], 0]) > 50 * MM)
    nbrs = [[] for _ in range(len(pos))]
    for i, j in conn:
        nbrs[i].append(j)
        nbrs[j].append(i)
    used, planted = set(), []
    for e in sorted(np.nonzero(axial)[0], key=lambda e: -abs(pos[conn[e, 0], 0])):
        a, b = int(conn[e, 0]), int(conn[e, 1])
        near = {a, b, *nbrs[a], *nbrs[b]}
        if near & used:
            continue
        planted.append((a, b, DELTAS[len(planted) % len(DELTAS)]))
        used |= near
        if len(planted) == 4 * len(DELTAS):
            break
    for a, b, d in planted:
        st = snot * (1.0 + d)
        xab = pos[b] - pos[a]
        cur_b = (pos[a] + disp[a]) + (R @ xab) * (1.0 + st)
        disp[b] = cur_b - pos[b]
    s.disp = disp
    cfg = dict(dt=1e-12, timesteps=1, enable_fracture=1, self_contact=0, allow_damping=0, allow_friction=0)
    return s, cfg, planted, snot


def _broken(sim, s):
    now = {tuple(x) for x in sim.connectivity(0).tolist()}
    return {tuple(x) for x in s.conn.tolist()} - now


@pytest.mark.parametrize("theta", [0.0, 0.6, 1.3])
def test_far_end_breaking_decisions_equal_fp64(theta):
    s, cfg, planted, snot = bar_with_planted_bonds(theta)
    assert len(planted) >= 3 * len(DELTAS)
    # the planted stretches, in FP64 as the reference computes them
    for a, b, d in planted:
        xi = s.pos[b] - s.pos[a]
        eta = (s.disp[b] - s.disp[a]) + xi
        st = (np.linalg.norm(eta) - np.linalg.norm(xi)) / np.linalg.norm(xi)
        assert abs(st / snot - 1.0 - d) < 1e-9, (d, st / snot - 1.0)
    want = {(min(a, b), max(a, b)) for a, b, d in planted if d > 0}
    got = {}
    for precision in ("fp64", "fp32c"):
        sim = Sim(s, cfg, precision)
        sim.step(1)
        got[precision] = _broken(sim, s)
        sim.close()
    assert got["fp64"] == want
    assert got["fp32c"] == want
