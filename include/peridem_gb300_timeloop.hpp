/*
 * peridem_gb300_timeloop.hpp -- the GB300 engine behind PeriDEM's own time-loop call.
 *
 * PeriDEM's driver (run/simulate3d.cpp:107-143) loads the particles, applies main.conf to the
 * Timeloop, Contact and RectWall objects and calls
 *     run_timeloop<dim>(PArr, TL, CN, Wall, CFGV);            (src/particle/timeloop.h:231-965)
 * A maintainer swaps the loop for the engine by including this header after PeriDEM's headers
 * (particle/particle2.h, particle/contact.h, particle/timeloop.h, read/read_config.h) and calling
 *     run_timeloop_gpu<dim>(PArr, TL, CN, Wall, CFGV);
 * in its place, then linking libperidem_gb300.so. The engine runs the configured loop with the
 * same output files (tc_%05u.h5, wall_%05u.h5, plotinfo.h5 in CFGV.output_dir) and, like
 * run_timeloop, leaves the final state in PArr (disp, CurrPos, vel, acc, force, NbdArr).
 *
 * The adapter only moves data across the C-ABI of peridem_gb300.h: it flattens PArr in file
 * order into pd_setup_arrays (NbdArr back to i < j pairs as NbdArr2conn does, timeloop.h:20-44),
 * copies the ConfigVal fields of the same names into pd_config, and takes the contact
 * constants and walls from CN and Wall (already configured by apply_config; the engine applies
 * the same overrides again from the config, which leaves them unchanged). Errors are returned
 * as the engine's status codes (pd_global_error / pd_last_error hold the text); PeriDEM would
 * pass them to errout.
 */
#ifndef PERIDEM_GB300_TIMELOOP_HPP
#define PERIDEM_GB300_TIMELOOP_HPP

#include <cstring>
#include <string>
#include <vector>

#include "peridem_gb300.h"

// ConfigVal -> pd_config: the same field names (read_config.h:14-99).
inline pd_config pd_config_from(const ConfigVal &c) {
  pd_config g;
  pd_config_default(&g);
  g.timesteps = c.timesteps;
  g.modulo = c.modulo;
  g.dt = c.dt;
  g.is_parallel = c.is_parallel;
  g.do_resume = c.do_resume;
  g.wall_resume = c.wall_resume;
  g.resume_ind = c.resume_ind;
  g.save_file = c.save_file;
  g.enable_fracture = c.enable_fracture;
  g.nl_bdry_only = c.nl_bdry_only;
  g.allow_damping = c.allow_damping;
  g.allow_friction = c.allow_friction;
  g.normal_stiffness = c.normal_stiffness;
  g.damping_ratio = c.damping_ratio;
  g.friction_coefficient = c.friction_coefficient;
  g.new_snot = c.new_snot;
  g.self_contact = c.self_contact;
  g.self_contact_rad = c.self_contact_rad;
  g.enable_cohesion = c.enable_cohesion;
  g.cohesion_scaling = c.cohesion_scaling;
  g.enable_torque = c.enable_torque;
  g.set_torque_timestep = c.set_torque_timestep;
  g.set_fracture_timestep = c.set_fracture_timestep;
  g.set_self_contact_timestep = c.set_self_contact_timestep;
  g.set_zero_wall_speed_timestep = c.set_zero_wall_speed_timestep;
  g.set_damping_timestep = c.set_damping_timestep;
  g.set_movable_index = c.set_movable_index;
  g.set_movable_timestep = c.set_movable_timestep;
  g.set_stoppable_index = c.set_stoppable_index;
  g.set_stoppable_timestep = c.set_stoppable_timestep;
  g.reset_partzero_y = c.reset_partzero_y;
  g.reset_partzero_y_timestep = c.reset_partzero_y_timestep;
  g.wheel_rad = c.wheel_rad;
  g.particle_w_fixed_velocity = c.particle_w_fixed_velocity;
  g.set_fix_velocity_timestep = c.set_fix_velocity_timestep;
  g.fix_velocity_angular = c.fix_velocity_angular;
  g.prescribed_angular_vel = c.prescribed_angular_vel;
  g.fix_velocity_mean_x = c.fix_velocity_mean_x;
  g.prescribed_velocity_mean_x = c.prescribed_velocity_mean_x;
  g.wall_left = c.wall_left;
  g.wall_right = c.wall_right;
  g.wall_top = c.wall_top;
  g.wall_bottom = c.wall_bottom;
  g.wall_x_min = c.wall_x_min;
  g.wall_y_min = c.wall_y_min;
  g.wall_z_min = c.wall_z_min;
  g.wall_x_max = c.wall_x_max;
  g.wall_y_max = c.wall_y_max;
  g.wall_z_max = c.wall_z_max;
  g.speed_wall_left = c.speed_wall_left;
  g.speed_wall_right = c.speed_wall_right;
  g.speed_wall_top = c.speed_wall_top;
  g.speed_wall_bottom = c.speed_wall_bottom;
  g.speed_wall_x_min = c.speed_wall_x_min;
  g.speed_wall_y_min = c.speed_wall_y_min;
  g.speed_wall_z_min = c.speed_wall_z_min;
  g.speed_wall_x_max = c.speed_wall_x_max;
  g.speed_wall_y_max = c.speed_wall_y_max;
  g.speed_wall_z_max = c.speed_wall_z_max;
  g.brazil = c.brazil;
  g.brazil_reset_wall_bottom_freq = c.brazil_reset_wall_bottom_freq;
  g.brazil_nonzero_wall_bottom_speed_freq = c.brazil_nonzero_wall_bottom_speed_freq;
  g.brazil_reset_wall_bottom_y = c.brazil_reset_wall_bottom_y;
  g.forcefield_type = c.forcefield_type;
  g.forcefield_scaling = c.forcefield_scaling;
  g.gradient_extforce = c.gradient_extforce;
  g.extforce_maxstep = c.extforce_maxstep;
  g.compute_wall_reaction = c.compute_wall_reaction;
  std::strncpy(g.setup_filename, c.setup_filename.c_str(), sizeof(g.setup_filename) - 1);
  std::strncpy(g.output_dir, c.output_dir.c_str(), sizeof(g.output_dir) - 1);
  return g;
}

// The flattened particles, kept alive while the engine reads them.
struct pd_flat_setup {
  std::vector<uint64_t> node_off{0}, conn_off{0}, bdry_off{0}, clamped_off{0};
  std::vector<double> pos, vol, disp, vel, acc, ext, delta, rho, cnot, snot, tval;
  std::vector<uint32_t> conn, bdry, clamped, taxis;
  std::vector<int32_t> mov, brk, stp;
  pd_setup_arrays su;
};

template <unsigned dim>
void pd_flatten(const std::vector<ParticleN<dim>> &PArr, const Contact &CN, RectWall<dim> &Wall, pd_flat_setup &f) {
  for (const auto &P : PArr) {
    for (unsigned i = 0; i < P.nnodes; ++i) {
      for (unsigned c = 0; c < 3; ++c) {
        f.pos.push_back(P.pos[i](c));
        f.disp.push_back(P.disp[i](c));
        f.vel.push_back(P.vel[i](c));
        f.acc.push_back(P.acc[i](c));
        f.ext.push_back(P.extforce[i](c));
      }
      f.vol.push_back(P.vol[i]);
    }
    for (unsigned i = 0; i < P.nnodes; ++i)  // NbdArr2conn (timeloop.h:20-44): i < q, row order
      for (unsigned q : P.NbdArr[i])
        if (i < q) {
          f.conn.push_back(i);
          f.conn.push_back(q);
        }
    for (unsigned b : P.boundary_nodes) f.bdry.push_back(b);
    for (unsigned b : P.clamped_nodes) f.clamped.push_back(b);
    f.node_off.push_back(f.node_off.back() + P.nnodes);
    f.conn_off.push_back(f.conn.size() / 2);
    f.bdry_off.push_back(f.bdry.size());
    f.clamped_off.push_back(f.clamped.size());
    f.delta.push_back(P.delta);
    f.rho.push_back(P.rho);
    f.cnot.push_back(P.cnot);
    f.snot.push_back(P.snot);
    f.tval.push_back(P.torque_val);
    f.taxis.push_back(P.torque_axis);
    f.mov.push_back(P.movable);
    f.brk.push_back(P.breakable);
    f.stp.push_back(P.stoppable);
  }
  pd_setup_arrays &s = f.su;
  std::memset(&s, 0, sizeof(s));
  s.n_particles = (uint32_t)PArr.size();
  s.node_offset = f.node_off.data();
  s.pos = f.pos.data();
  s.vol = f.vol.data();
  s.disp = f.disp.data();
  s.vel = f.vel.data();
  s.acc = f.acc.data();
  s.extforce = f.ext.data();
  s.conn_offset = f.conn_off.data();
  s.conn = f.conn.data();
  s.bdry_offset = f.bdry_off.data();
  s.bdry = f.bdry.data();
  s.clamped_offset = f.clamped_off.data();
  s.clamped = f.clamped.data();
  s.delta = f.delta.data();
  s.rho = f.rho.data();
  s.cnot = f.cnot.data();
  s.snot = f.snot.data();
  s.torque_val = f.tval.data();
  s.movable = f.mov.data();
  s.breakable = f.brk.data();
  s.stoppable = f.stp.data();
  s.torque_axis = f.taxis.data();
  s.contact_radius = CN.contact_rad;
  s.normal_stiffness = CN.normal_stiffness;
  s.damping_ratio = CN.damping_ratio;
  s.friction_coefficient = CN.friction_coefficient;
  s.allow_wall = Wall.allow_wall;
  const std::vector<double> w = Wall.lrtb();
  s.n_geom_wall = (int32_t)w.size();
  for (size_t k = 0; k < w.size() && k < 6; ++k) s.geom_wall_info[k] = w[k];
}

// run_timeloop<dim> on the GPU: the configured loop with its frames, the final state back in
// PArr. TL is accepted for the call's shape only: its fields come from CFGV (timeloop.h:184-225).
template <unsigned dim>
int run_timeloop_gpu(std::vector<ParticleN<dim>> &PArr, Timeloop TL, Contact CN, RectWall<dim> Wall,
                     ConfigVal CFGV, int precision = PD_FP64) {
  static_assert(dim == 3, "the engine runs the 3D time loop");
  (void)TL;
  pd_flat_setup f;
  pd_flatten<dim>(PArr, CN, Wall, f);
  pd_config cfg = pd_config_from(CFGV);
  pd_sim *sim = nullptr;
  int rc = pd_create_from_arrays(&f.su, &cfg, precision, &sim);
  if (rc != PD_OK) return rc;
  rc = pd_run(sim);
  if (rc == PD_OK) rc = pd_sync(sim, -1);
  if (rc == PD_OK) {  // the final state back into PArr, as run_timeloop leaves it
    const size_t N = f.vol.size();
    std::vector<double> cur(3 * N), vel(3 * N), acc(3 * N), force(3 * N), disp(3 * N);
    rc = pd_get_node_state(sim, cur.data(), vel.data(), acc.data(), force.data(), disp.data());
    std::vector<uint32_t> pairs;
    for (size_t p = 0; rc == PD_OK && p < PArr.size(); ++p) {
      auto &P = PArr[p];
      const size_t a = f.node_off[p];
      P.CurrPos.resize(P.nnodes);
      for (unsigned i = 0; i < P.nnodes; ++i)
        for (unsigned c = 0; c < 3; ++c) {
          P.CurrPos[i](c) = cur[3 * (a + i) + c];
          P.vel[i](c) = vel[3 * (a + i) + c];
          P.acc[i](c) = acc[3 * (a + i) + c];
          P.force[i](c) = force[3 * (a + i) + c];
          P.disp[i](c) = disp[3 * (a + i) + c];
        }
      uint64_t n = 0;
      rc = pd_get_connectivity(sim, (uint32_t)p, nullptr, 0, &n);
      if (rc != PD_OK) break;
      pairs.resize(2 * (n ? n : 1));
      rc = pd_get_connectivity(sim, (uint32_t)p, pairs.data(), n, &n);
      if (rc != PD_OK) break;
      // NbdArr from the live pairs (conn2NArr push order, load_hdf5.h:27-37)
      for (auto &row : P.NbdArr) row.clear();
      for (uint64_t l = 0; l < n; ++l) {
        P.NbdArr[pairs[2 * l]].push_back(pairs[2 * l + 1]);
        P.NbdArr[pairs[2 * l + 1]].push_back(pairs[2 * l]);
      }
    }
  }
  pd_close(sim);
  return rc;
}

#endif /* PERIDEM_GB300_TIMELOOP_HPP */
