// pd_sim.h -- the opaque handle behind pd_sim* of include/peridem_gb300.h.
#ifndef PD_SIM_H
#define PD_SIM_H
#include <string>

#include "pd_engine.h"

struct pd_sim {
  pdg::Engine eng;
  pd_config cfg;
  std::string outdir;
};

namespace pdg {
int host_sim_from_arrays(const pd_setup_arrays *su, const pd_config *cfg, HostSim &hs, std::string &err);
// Records the text pd_global_error() returns (thread-local) and passes rc through.
int set_global_error(int rc, const std::string &msg);
}

#endif
