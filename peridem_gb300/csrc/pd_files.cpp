// pd_files.cpp -- file boundary (setup.h5 in, plotinfo/tc/wall frames out).
#include <string>

#include "pd_sim.h"

extern "C" {

int pd_open(const char *conf, const char *setup_h5, const char *outdir, int precision, pd_sim **out) {
  (void)conf;
  (void)setup_h5;
  (void)outdir;
  (void)precision;
  if (out) *out = nullptr;
  return PD_EIO;
}

int pd_run(pd_sim *sim) {
  (void)sim;
  return PD_EIO;
}

int pd_write_frame(pd_sim *sim, uint32_t counter) {
  (void)sim;
  (void)counter;
  return PD_EIO;
}

}  // extern "C"
