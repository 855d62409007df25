// pd_config.cpp -- the `main.conf` grammar (src/read/read_config.h:14-435).
//
// Same keys, defaults and sentinels as ConfigVal. Each line has all whitespace removed,
// lines starting with '#' and empty lines are skipped, the text before the first '=' is
// the key and the rest is the value. Integer keys go through std::stoi, real keys through
// std::stod; boolean keys keep stoi(value) != 0, as assigning an int to a C++ bool does.
// An unknown key prints "[Error]: Wrong config name: <key> !!" to stderr and parsing goes
// on (read_config.h:425-427). Where the reference would abort on an uncaught exception
// (a missing value, a non-numeric value) this parser returns PD_ECONFIG instead.
#include <cctype>
#include <cstddef>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>

#include "peridem_gb300.h"

namespace {

enum Kind { K_U32, K_I32, K_BOOL, K_F64, K_F32 };

struct Key {
  const char *name;
  Kind kind;
  size_t off;
};

#define PD_KEY(field, kind) {#field, kind, offsetof(pd_config, field)}

const Key kKeys[] = {
    PD_KEY(timesteps, K_U32),
    PD_KEY(modulo, K_U32),
    PD_KEY(dt, K_F64),
    PD_KEY(is_parallel, K_BOOL),
    PD_KEY(do_resume, K_BOOL),
    PD_KEY(wall_resume, K_BOOL),
    PD_KEY(resume_ind, K_U32),
    PD_KEY(save_file, K_BOOL),
    PD_KEY(enable_fracture, K_BOOL),
    PD_KEY(nl_bdry_only, K_BOOL),
    PD_KEY(particle_w_fixed_velocity, K_I32),
    PD_KEY(set_fix_velocity_timestep, K_I32),
    PD_KEY(fix_velocity_angular, K_BOOL),
    PD_KEY(prescribed_angular_vel, K_F64),
    PD_KEY(fix_velocity_mean_x, K_BOOL),
    PD_KEY(prescribed_velocity_mean_x, K_F64),
    PD_KEY(allow_damping, K_BOOL),
    PD_KEY(allow_friction, K_BOOL),
    PD_KEY(damping_ratio, K_F64),
    PD_KEY(friction_coefficient, K_F64),
    PD_KEY(normal_stiffness, K_F64),
    PD_KEY(new_snot, K_F64),
    PD_KEY(forcefield_type, K_I32),
    PD_KEY(forcefield_scaling, K_F64),
    PD_KEY(self_contact, K_BOOL),
    PD_KEY(self_contact_rad, K_F64),
    PD_KEY(enable_torque, K_BOOL),
    PD_KEY(set_torque_timestep, K_I32),
    PD_KEY(set_fracture_timestep, K_I32),
    PD_KEY(set_self_contact_timestep, K_I32),
    PD_KEY(set_damping_timestep, K_I32),
    PD_KEY(set_zero_wall_speed_timestep, K_I32),
    PD_KEY(enable_cohesion, K_BOOL),
    PD_KEY(cohesion_scaling, K_F64),
    PD_KEY(set_movable_index, K_I32),
    PD_KEY(set_movable_timestep, K_I32),
    PD_KEY(set_stoppable_index, K_I32),
    PD_KEY(set_stoppable_timestep, K_I32),
    PD_KEY(reset_partzero_y, K_BOOL),
    PD_KEY(reset_partzero_y_timestep, K_U32),
    PD_KEY(wheel_rad, K_F64),
    PD_KEY(wall_left, K_F64),
    PD_KEY(wall_right, K_F64),
    PD_KEY(wall_top, K_F64),
    PD_KEY(wall_bottom, K_F64),
    PD_KEY(speed_wall_left, K_F64),
    PD_KEY(speed_wall_right, K_F64),
    PD_KEY(speed_wall_top, K_F64),
    PD_KEY(speed_wall_bottom, K_F64),
    PD_KEY(brazil, K_BOOL),
    PD_KEY(brazil_reset_wall_bottom_freq, K_I32),
    PD_KEY(brazil_nonzero_wall_bottom_speed_freq, K_I32),
    PD_KEY(brazil_reset_wall_bottom_y, K_F32),
    PD_KEY(wall_x_min, K_F64),
    PD_KEY(wall_y_min, K_F64),
    PD_KEY(wall_z_min, K_F64),
    PD_KEY(wall_x_max, K_F64),
    PD_KEY(wall_y_max, K_F64),
    PD_KEY(wall_z_max, K_F64),
    PD_KEY(speed_wall_x_min, K_F64),
    PD_KEY(speed_wall_y_min, K_F64),
    PD_KEY(speed_wall_z_min, K_F64),
    PD_KEY(speed_wall_x_max, K_F64),
    PD_KEY(speed_wall_y_max, K_F64),
    PD_KEY(speed_wall_z_max, K_F64),
    PD_KEY(gradient_extforce, K_BOOL),
    PD_KEY(extforce_maxstep, K_U32),
    PD_KEY(compute_wall_reaction, K_BOOL),
};
#undef PD_KEY

}  // namespace

extern "C" int pd_config_default(pd_config *c) {
  if (!c) return PD_EINVAL;
  std::memset(c, 0, sizeof(*c));
  // ConfigVal() (read_config.h:102-167) and in-class initialisers (read_config.h:36-99)
  c->timesteps = 8000;
  c->modulo = 100;
  c->dt = 0.02 / 1e5;
  c->is_parallel = 1;
  c->do_resume = 0;
  c->wall_resume = 0;
  c->resume_ind = 50;
  c->save_file = 1;
  c->enable_fracture = 0;
  c->nl_bdry_only = 0;
  c->allow_damping = 1;
  c->allow_friction = 1;
  c->self_contact = 1;
  c->self_contact_rad = -1;
  c->enable_cohesion = 0;
  c->cohesion_scaling = 1;
  c->enable_torque = 0;
  c->set_torque_timestep = -1;
  c->set_fracture_timestep = -1;
  c->set_self_contact_timestep = -1;
  c->set_zero_wall_speed_timestep = -1;
  c->set_damping_timestep = -1;
  c->set_movable_index = -1;
  c->set_movable_timestep = -1;
  c->set_stoppable_index = -1;
  c->set_stoppable_timestep = -1;
  c->reset_partzero_y = 0;
  c->reset_partzero_y_timestep = 0;
  c->wheel_rad = 0;
  c->particle_w_fixed_velocity = -1;
  c->set_fix_velocity_timestep = -1;
  c->fix_velocity_angular = 0;
  c->prescribed_angular_vel = -999;
  c->fix_velocity_mean_x = 0;
  c->prescribed_velocity_mean_x = -999;
  c->normal_stiffness = -1;
  c->damping_ratio = -1;
  c->friction_coefficient = -1;
  c->new_snot = -1;
  c->wall_left = c->wall_right = c->wall_top = c->wall_bottom = -999;
  c->wall_x_min = c->wall_y_min = c->wall_z_min = -999;
  c->wall_x_max = c->wall_y_max = c->wall_z_max = -999;
  c->speed_wall_left = c->speed_wall_right = c->speed_wall_top = c->speed_wall_bottom = 0;
  c->brazil = 0;
  c->brazil_reset_wall_bottom_freq = -1;
  c->brazil_nonzero_wall_bottom_speed_freq = -1;
  c->brazil_reset_wall_bottom_y = -999;
  c->speed_wall_x_min = c->speed_wall_y_min = c->speed_wall_z_min = 0;
  c->speed_wall_x_max = c->speed_wall_y_max = c->speed_wall_z_max = 0;
  c->forcefield_type = 0;
  c->forcefield_scaling = 1e9;
  c->gradient_extforce = 0;
  c->extforce_maxstep = 0;
  c->compute_wall_reaction = 0;
  std::strncpy(c->setup_filename, "data/hdf5/all.h5", sizeof(c->setup_filename) - 1);
  std::strncpy(c->output_dir, "output/hdf5/", sizeof(c->output_dir) - 1);
  c->n_unknown_keys = 0;
  return PD_OK;
}

extern "C" int pd_config_read(const char *path, pd_config *c) {
  if (!path || !c) return PD_EINVAL;
  std::ifstream f(path);
  if (!f.is_open()) {
    std::cerr << "Couldn't open config file for reading.\n";
    return PD_ECONFIG;
  }
  std::cout << "Reading config file: " << path << std::endl;
  std::string line;
  int rc = PD_OK;
  while (std::getline(f, line)) {
    std::string s;
    for (char ch : line)
      if (!std::isspace((unsigned char)ch)) s.push_back(ch);
    if (s.empty() || s[0] == '#') continue;
    size_t eq = s.find('=');
    std::string name = s.substr(0, eq);
    std::string value = (eq == std::string::npos) ? s : s.substr(eq + 1);
    if (value.empty()) std::cout << "[Error] Missing value for option: " << name << std::endl;
    const Key *k = nullptr;
    for (const Key &kk : kKeys)
      if (name == kk.name) {
        k = &kk;
        break;
      }
    if (!k) {
      std::cerr << "[Error]: Wrong config name: " << name << " !!\n";
      c->n_unknown_keys++;
      continue;
    }
    char *base = reinterpret_cast<char *>(c) + k->off;
    try {
      switch (k->kind) {
        case K_U32: *reinterpret_cast<uint32_t *>(base) = (uint32_t)std::stoi(value); break;
        case K_I32: *reinterpret_cast<int32_t *>(base) = (int32_t)std::stoi(value); break;
        case K_BOOL: *reinterpret_cast<int32_t *>(base) = std::stoi(value) != 0 ? 1 : 0; break;
        case K_F64: *reinterpret_cast<double *>(base) = std::stod(value); break;
        case K_F32: *reinterpret_cast<double *>(base) = (double)(float)std::stod(value); break;
      }
    } catch (const std::exception &) {
      std::cerr << "[Error]: bad value for config name: " << name << "\n";
      rc = PD_ECONFIG;
    }
  }
  std::cout << "Reading config file: Done" << std::endl;
  return rc;
}
