"""Small seeded cases shared by the parity tests (sizes the oracle finishes in seconds)."""
from __future__ import annotations

import numpy as np

from peridem_gb300 import gen

MM = 1e-3


def impact_walls(steps=60):
    """Two small spheres, one moving, inside a tight wall box: contact, walls, fracture,
    self-contact after breaking."""
    s, cfg = gen.two_sphere(R=0.3 * MM, h=0.1 * MM, v=20.0, steps=steps, walls=True)
    cfg.update(compute_wall_reaction=1)
    return s, cfg


def impact_free(steps=40):
    """The same pair without walls, sphere B fast enough to break bonds on impact."""
    s, cfg = gen.two_sphere(R=0.4 * MM, h=0.1 * MM, v=60.0, gap=0.1, steps=steps, walls=False)
    return s, cfg


def cubes_gravity(steps=40, n=2):
    """n^3 rotated cubes with gravity, extforce and walls (cubes125 in miniature)."""
    s, cfg = gen.cubes125(n=n, edge=0.5 * MM, h=0.125 * MM, steps=steps, gap=0.05 * MM, g=9.81e6)
    cfg.update(compute_wall_reaction=1)
    return s, cfg


def toggles(steps=30):
    """Scheduled toggles, a fixed particle made movable mid-run, clamped nodes, torque,
    gradient extforce and a moving wall."""
    s, cfg = gen.two_sphere(R=0.3 * MM, h=0.1 * MM, v=15.0, steps=steps, walls=True)
    s.movable[0] = 0
    s.stoppable[0] = 1
    s.torque_val[1] = 1e9
    s.torque_axis[1] = 1
    # clamp a few nodes of particle 1
    n1 = s.particle_slice(1).stop - s.particle_slice(1).start
    cl = np.array([0, 3, n1 - 1], dtype=np.uint32)
    s.clamped_offset = np.array([0, 0, len(cl)], dtype=np.uint64)
    s.clamped = cl
    s.extforce[:] = [0.0, 0.0, -2.4e7]
    cfg.update(set_movable_index=0, set_movable_timestep=7, set_torque_timestep=5, gradient_extforce=1,
               extforce_maxstep=12, set_zero_wall_speed_timestep=20, speed_wall_x_max=-3.0,
               speed_wall_z_min=0.5, set_damping_timestep=3, allow_damping=0, compute_wall_reaction=1)
    return s, cfg


def bdry_only(steps=30):
    """nl_bdry_only = 1: contact and walls only between boundary-node lists."""
    s, cfg = gen.two_sphere(R=0.3 * MM, h=0.1 * MM, v=20.0, steps=steps, walls=True)
    cfg.update(nl_bdry_only=1, compute_wall_reaction=1)
    return s, cfg


def prescribed(steps=30):
    """Prescribed velocity of particle 0 (mean x velocity and angular velocity about z, from
    step 4 on), and reset_partzero_y moving particle 0 above the other particle at step 9."""
    s, cfg = gen.two_sphere(R=0.3 * MM, h=0.1 * MM, v=15.0, steps=steps, walls=True)
    cfg.update(particle_w_fixed_velocity=0, set_fix_velocity_timestep=4, fix_velocity_mean_x=1,
               prescribed_velocity_mean_x=-2.5, fix_velocity_angular=1, prescribed_angular_vel=2.0e4,
               reset_partzero_y=1, reset_partzero_y_timestep=9, wheel_rad=0.35 * MM, compute_wall_reaction=1)
    return s, cfg


def notched(steps=45):
    """Config 3 in miniature: steel plate with two edge notches hit by an unbreakable block."""
    s, cfg = gen.notched_plate(Lx=6.0 * MM, Ly=8.0 * MM, Lz=1.5 * MM, h=0.5 * MM, notch_len=3.0 * MM,
                               notch_x=(2.0 * MM, 4.0 * MM), imp_w=2.0 * MM, imp_len=1.5 * MM, v=150.0,
                               steps=steps, dt=2e-8, gap=-0.6)
    return s, cfg


CASES = {
    "impact_walls": impact_walls,
    "impact_free": impact_free,
    "cubes_gravity": cubes_gravity,
    "toggles": toggles,
    "bdry_only": bdry_only,
    "prescribed": prescribed,
    "notched": notched,
}
