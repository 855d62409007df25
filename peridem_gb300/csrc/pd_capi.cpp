// pd_capi.cpp -- the extern "C" entry points of include/peridem_gb300.h over pdg::Engine.
#include <cstring>
#include <string>

#include "pd_engine.h"
#include "pd_sim.h"

namespace {
thread_local std::string g_error;

int fail_global(int rc, const std::string &msg) {
  g_error = msg;
  return rc;
}
}  // namespace

namespace pdg {

int set_global_error(int rc, const std::string &msg) { return fail_global(rc, msg); }

// Reads caller arrays into a HostSim (the particle vector the reference loads in
// load_particles<3>, load_hdf5.h:41-113).
int host_sim_from_arrays(const pd_setup_arrays *su, const pd_config *cfg, HostSim &hs, std::string &err) {
  if (!su || !cfg) {
    err = "null setup or config";
    return PD_EINVAL;
  }
  if (su->n_particles == 0 || !su->node_offset || !su->pos || !su->vol || !su->disp || !su->vel || !su->acc ||
      !su->extforce || !su->conn_offset || !su->delta || !su->rho || !su->cnot || !su->snot || !su->torque_val ||
      !su->movable || !su->breakable || !su->stoppable || !su->torque_axis) {
    err = "setup arrays incomplete";
    return PD_EINVAL;
  }
  const uint32_t np = su->n_particles;
  if (su->node_offset[0] != 0 || su->conn_offset[0] != 0) {
    err = "node_offset/conn_offset must start at 0";
    return PD_EINVAL;
  }
  for (uint32_t p = 0; p < np; ++p) {
    if (su->node_offset[p + 1] <= su->node_offset[p]) {
      err = "particle " + std::to_string(p) + " has no nodes";
      return PD_EINVAL;
    }
    if (su->conn_offset[p + 1] < su->conn_offset[p]) {
      err = "conn_offset not monotone";
      return PD_EINVAL;
    }
    if (su->torque_axis[p] > 2) {
      err = "torque_axis above 2";
      return PD_EINVAL;
    }
    if (!(su->rho[p] > 0)) {
      err = "rho must be positive";
      return PD_EINVAL;
    }
  }
  if (!(su->contact_radius > 0)) {
    err = "contact_radius must be positive";
    return PD_EINVAL;
  }
  const uint64_t N = su->node_offset[np];
  const uint64_t M = su->conn_offset[np];
  hs.cfg = *cfg;
  hs.np = np;
  hs.node_offset.assign(su->node_offset, su->node_offset + np + 1);
  hs.pos.assign(su->pos, su->pos + 3 * N);
  // read only while the engine is built, which happens before the creating call returns
  hs.vol.view(su->vol, N);
  hs.disp.view(su->disp, 3 * N);
  hs.vel.view(su->vel, 3 * N);
  hs.acc.view(su->acc, 3 * N);
  hs.ext.view(su->extforce, 3 * N);
  hs.conn_offset.assign(su->conn_offset, su->conn_offset + np + 1);
  if (M) {
    if (!su->conn) {
      err = "conn missing";
      return PD_EINVAL;
    }
    hs.conn.view(su->conn, 2 * M);
  }
  if (su->bdry_offset && su->bdry) {
    hs.bdry_offset.assign(su->bdry_offset, su->bdry_offset + np + 1);
    hs.bdry.assign(su->bdry, su->bdry + su->bdry_offset[np]);
  }
  if (su->clamped_offset && su->clamped) {
    hs.clamped_offset.assign(su->clamped_offset, su->clamped_offset + np + 1);
    hs.clamped.assign(su->clamped, su->clamped + su->clamped_offset[np]);
  }
  for (uint32_t p = 0; p < np; ++p) {
    uint64_t nloc = su->node_offset[p + 1] - su->node_offset[p];
    if (!hs.bdry_offset.empty())
      for (uint64_t l = hs.bdry_offset[p]; l < hs.bdry_offset[p + 1]; ++l)
        if (hs.bdry[l] >= nloc) {
          err = "bdry_nodes index out of range";
          return PD_EINVAL;
        }
    if (!hs.clamped_offset.empty())
      for (uint64_t l = hs.clamped_offset[p]; l < hs.clamped_offset[p + 1]; ++l)
        if (hs.clamped[l] >= nloc) {
          err = "clamped_nodes index out of range";
          return PD_EINVAL;
        }
  }
  hs.delta.assign(su->delta, su->delta + np);
  hs.rho.assign(su->rho, su->rho + np);
  hs.cnot.assign(su->cnot, su->cnot + np);
  hs.snot.assign(su->snot, su->snot + np);
  hs.tval.assign(su->torque_val, su->torque_val + np);
  hs.movable.assign(su->movable, su->movable + np);
  hs.breakable.assign(su->breakable, su->breakable + np);
  hs.stoppable.assign(su->stoppable, su->stoppable + np);
  hs.taxis.assign(su->torque_axis, su->torque_axis + np);
  hs.Rc = su->contact_radius;
  hs.Kn = su->normal_stiffness;
  hs.zeta = su->damping_ratio;
  hs.mu = su->friction_coefficient;
  hs.allow_wall = su->allow_wall;
  hs.n_geom_wall = su->n_geom_wall;
  for (int k = 0; k < 6; ++k) hs.geom[k] = su->geom_wall_info[k];
  return PD_OK;
}

}  // namespace pdg

extern "C" {

const char *pd_global_error(void) { return g_error.c_str(); }

int pd_create_from_arrays(const pd_setup_arrays *setup, const pd_config *cfg, int precision, pd_sim **out) {
  if (!out) return fail_global(PD_EINVAL, "null output handle");
  *out = nullptr;
  if (precision != PD_FP64 && precision != PD_FP32C) return fail_global(PD_EINVAL, "unknown precision form");
  std::vector<pdg::HostSim> sims(1);
  std::string err;
  int rc = pdg::host_sim_from_arrays(setup, cfg, sims[0], err);
  if (rc != PD_OK) return fail_global(rc, err);
  pd_sim *s = new pd_sim();
  s->cfg = *cfg;
  s->outdir = cfg->output_dir;  // frames go where the config says (ConfigVal::output_dir)
  rc = s->eng.init(sims, precision);
  if (rc != PD_OK) {
    std::string e = s->eng.err;
    delete s;
    return fail_global(rc, e);
  }
  *out = s;
  return PD_OK;
}

int pd_step(pd_sim *s, uint32_t nsteps) {
  if (!s) return fail_global(PD_EINVAL, "null handle");
  return s->eng.step(nsteps);
}

int pd_sync(pd_sim *s, int timeout_ms) {
  if (!s) return fail_global(PD_EINVAL, "null handle");
  return s->eng.sync(timeout_ms);
}

int pd_set_stream(pd_sim *s, void *stream) {
  if (!s) return fail_global(PD_EINVAL, "null handle");
  return s->eng.set_stream((cudaStream_t)stream);
}

int pd_num_nodes(const pd_sim *s, uint64_t *n_nodes, uint32_t *n_particles) {
  if (!s) return fail_global(PD_EINVAL, "null handle");
  if (n_nodes) *n_nodes = s->eng.num_nodes();
  if (n_particles) *n_particles = s->eng.num_particles();
  return PD_OK;
}

int pd_get_state(pd_sim *s, double *curpos, double *vel, double *acc, double *force) {
  if (!s) return fail_global(PD_EINVAL, "null handle");
  return s->eng.get_state(curpos, vel, acc, force, nullptr);
}

int pd_get_applied_force_density(pd_sim *s, double *afd) {
  if (!s || !afd) return fail_global(PD_EINVAL, "null argument");
  return s->eng.get_afd(afd);
}

int pd_get_damage(pd_sim *s, double *damage) {
  if (!s || !damage) return fail_global(PD_EINVAL, "null argument");
  return s->eng.get_damage(damage);
}

int pd_get_disp(pd_sim *s, double *disp) {
  if (!s) return fail_global(PD_EINVAL, "null handle");
  return s->eng.get_state(nullptr, nullptr, nullptr, nullptr, disp);
}

int pd_get_node_state(pd_sim *s, double *curpos, double *vel, double *acc, double *force, double *disp) {
  if (!s) return fail_global(PD_EINVAL, "null handle");
  return s->eng.get_state(curpos, vel, acc, force, disp);
}

int pd_set_state(pd_sim *s, const double *disp, const double *vel, const double *acc) {
  if (!s) return fail_global(PD_EINVAL, "null handle");
  return s->eng.set_state(disp, vel, acc);
}

int pd_get_connectivity(pd_sim *s, uint32_t particle, uint32_t *pairs, uint64_t cap, uint64_t *n) {
  if (!s || !n) return fail_global(PD_EINVAL, "null argument");
  return s->eng.get_connectivity(particle, pairs, cap, n);
}

int pd_get_wall(pd_sim *s, double *wall_info, double *reaction) {
  if (!s) return fail_global(PD_EINVAL, "null handle");
  return s->eng.get_wall(0, wall_info, reaction);
}

int pd_get_aabb(pd_sim *s, double *lrtb) {
  if (!s || !lrtb) return fail_global(PD_EINVAL, "null argument");
  return s->eng.get_aabb(lrtb);
}

int pd_get_stats(pd_sim *s, pd_stats *st) {
  if (!s || !st) return fail_global(PD_EINVAL, "null argument");
  return s->eng.get_stats(st);
}

const char *pd_last_error(const pd_sim *s) {
  if (!s) return g_error.c_str();
  return s->eng.err.c_str();
}

int pd_close(pd_sim *s) {
  if (!s) return PD_OK;
  delete s;
  return PD_OK;
}

int pd_set_tuning(pd_sim *s, double skin_frac, uint32_t cand_cap, int threads_per_block, int stats,
                  int use_graphs) {
  if (!s) return fail_global(PD_EINVAL, "null handle");
  return s->eng.set_tuning(skin_frac, cand_cap, threads_per_block, stats, use_graphs);
}

int pd_clear_device_errors(pd_sim *s) {
  if (!s) return fail_global(PD_EINVAL, "null handle");
  return s->eng.clear_device_errors();
}

double pd_step_bytes(const pd_sim *s) {
  if (!s) return 0.0;
  return s->eng.step_bytes(s->eng.initial_bonds());
}

}  // extern "C"

extern "C" {

int pd_profile_steps(pd_sim *s, uint32_t nsteps, double *phase_ms) {
  if (!s || !phase_ms) return fail_global(PD_EINVAL, "null argument");
  for (int i = 0; i < 4; ++i) phase_ms[i] = 0.0;
  return s->eng.profile(nsteps, phase_ms);
}

int pd_count_live_bonds(pd_sim *s, uint64_t *live) {
  if (!s || !live) return fail_global(PD_EINVAL, "null argument");
  return s->eng.count_live_bonds(live);
}

}  // extern "C"

extern "C" {

int pd_autotune(pd_sim *s, uint32_t steps_per_variant, int *chosen, double *variant_ms) {
  if (!s) return fail_global(PD_EINVAL, "null handle");
  return s->eng.autotune(steps_per_variant, chosen, variant_ms);
}

int pd_set_variant(pd_sim *s, int variant) {
  if (!s) return fail_global(PD_EINVAL, "null handle");
  return s->eng.set_variant(variant);
}

int pd_num_variants(void) { return pdg::num_bond_variants(); }

int pd_set_persist_lanes(pd_sim *s, int lanes) {
  if (!s) return fail_global(PD_EINVAL, "null handle");
  return s->eng.set_persist_lanes(lanes);
}

int pd_persist_lanes(const pd_sim *s) { return s ? s->eng.persist_lanes() : -1; }

int pd_graph_mode(const pd_sim *s) { return s ? s->eng.graph_mode() : -1; }

int pd_snapshot(pd_sim *s) {
  if (!s) return fail_global(PD_EINVAL, "null handle");
  return s->eng.snapshot();
}

int pd_restore(pd_sim *s) {
  if (!s) return fail_global(PD_EINVAL, "null handle");
  return s->eng.restore();
}

}  // extern "C"
