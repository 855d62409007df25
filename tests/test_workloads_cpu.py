"""Workload generators (no GPU): the bench's bounded CPU sample of config 2 is built as the first
particles of the same packing, without generating the whole packing."""
import numpy as np

from peridem_gb300 import gen


def test_crush_count_is_the_first_particles_of_the_packing():
    full, cfg_full = gen.crush512(n=4)
    part, cfg_part = gen.crush512(n=4, count=8)
    sub = full.subset(list(range(8)))
    for k in ("pos", "vol", "conn", "node_offset", "conn_offset", "disp", "vel", "acc", "extforce", "bdry",
              "bdry_offset", "rho", "cnot", "snot", "delta", "geom_wall_info"):
        np.testing.assert_array_equal(getattr(part, k), getattr(sub, k), err_msg=k)
    for k in ("contact_radius", "normal_stiffness", "damping_ratio", "friction_coefficient", "allow_wall"):
        assert getattr(part, k) == getattr(sub, k), k
    assert cfg_part == cfg_full


def test_crush_4m_scales_the_lattice_and_the_step():
    s, cfg = gen.crush512_4m(count=2)
    assert cfg["dt"] == 3e-9
    assert all(np.isclose(h, [0.03e-3, 0.045e-3, 0.06e-3]).any() for h in s.meta["h"])
    assert np.isclose(s.contact_radius, 0.5 * 0.03e-3)
