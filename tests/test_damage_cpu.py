"""The damage field's oracle (oracle.damage, restating plot3d_timestep.py:95-105, 108-117 and
156-166 of examples/3D-HPC-aggregate-particle-breakage): known answers on small
Connectivities and the golden frames PeriDEM's own code wrote."""
from types import SimpleNamespace

import numpy as np

from oracle import oracle as O
from tests.golden.make_golden import load


def _setup(n_nodes, conns):
    node_offset = np.concatenate([[0], np.cumsum(n_nodes)]).astype(np.uint64)
    conn_offset = np.concatenate([[0], np.cumsum([len(c) for c in conns])]).astype(np.uint64)
    conn = np.concatenate([np.asarray(c, dtype=np.uint32).reshape(-1, 2) for c in conns])
    return SimpleNamespace(n_particles=len(n_nodes), node_offset=node_offset, conn_offset=conn_offset, conn=conn)


def test_damage_known_answers():
    # particle 0: a triangle that loses (0, 2); particle 1: node 2 never had a bond
    s = _setup([3, 3], [[(0, 1), (0, 2), (1, 2)], [(0, 1)]])
    d = O.damage(s, [np.array([(0, 1), (1, 2)]), np.array([(0, 1)])])
    np.testing.assert_array_equal(d[:5], [0.5, 0.0, 0.5, 0.0, 0.0])
    assert np.isnan(d[5])
    # every bond broken: damage 1 wherever there were bonds
    d = O.damage(s, [np.zeros((0, 2)), np.zeros((0, 2))])
    np.testing.assert_array_equal(d[:5], 1.0)


def _loop_damage(conn_setup, conn_now, n):
    """The plotting script's own loop, element by element."""
    orig, now = np.zeros(n), np.zeros(n)
    for i, j in conn_setup:
        orig[i] += 1
        orig[j] += 1
    for i, j in conn_now:
        now[i] += 1
        now[j] += 1
    with np.errstate(invalid="ignore", divide="ignore"):
        return (orig - now) / orig


def test_damage_of_golden_frames():
    g = load("impact_walls")
    s = g["setup"]
    for counter, f in g["frames"].items():
        co = f["conn_offset"]
        conns = [f["conn"][co[p]:co[p + 1]] for p in range(s.n_particles)]
        d = O.damage(s, conns)
        ref = np.concatenate([
            _loop_damage(s.conn[int(s.conn_offset[p]):int(s.conn_offset[p + 1])], conns[p],
                         int(s.node_offset[p + 1] - s.node_offset[p])) for p in range(s.n_particles)])
        np.testing.assert_array_equal(d, ref, err_msg=f"frame {counter}")
        ok = ~np.isnan(d)
        assert ((d[ok] >= 0) & (d[ok] <= 1)).all()
        assert d[ok].max() > 0, "the golden frames have broken bonds"
