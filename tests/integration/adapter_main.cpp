// TEST INFRASTRUCTURE: PeriDEM's driver steps (run/simulate3d.cpp:37-143) with the time loop
// replaced by run_timeloop_gpu (include/peridem_gb300_timeloop.hpp). Built by `make -C oracle
// adapter` against the reference's own headers and the stand-in Eigen / MPI / HDF5 headers of
// oracle/ref_shim, to check that the adapter binds to the reference's types and to the
// engine's C-ABI (compiled and linked; running it needs a GPU and the reference sources on the
// same machine).
#define EIGEN_DONT_PARALLELIZE
#include <cstdio>
#include <string>

#include "Eigen/Dense"
using namespace Eigen;
#include <mpi.h>

// the reference's headers in its driver's order (they rely on it)
#include "read/load_hdf5.h"
#include "read/read_config.h"
#include "particle/timeloop.h"
#include "peridem_gb300_timeloop.hpp"

int main(int argc, char *argv[]) {
  if (argc < 4) {
    std::printf("usage: %s main.conf setup.h5 outdir [fp32c]\n", argv[0]);
    return 0;
  }
  MPI_Init(&argc, &argv);
  ConfigVal CFGV;
  CFGV.setup_filename = argv[2];
  CFGV.output_dir = argv[3];
  CFGV.read_file(argv[1]);
  auto PArr = load_particles<3>(CFGV);
  Contact CN = load_contact(CFGV);
  RectWall<3> Wall = load_wall<3>(CFGV);
  Timeloop TL(100);
  TL.apply_config(CFGV);
  CN.apply_config(CFGV);
  Wall.apply_config(CFGV);
  for (unsigned i = 0; i < PArr.size(); i++) PArr[i].break_bonds = 1;
  const int precision = (argc > 4 && std::string(argv[4]) == "fp32c") ? PD_FP32C : PD_FP64;
  const int rc = run_timeloop_gpu<3>(PArr, TL, CN, Wall, CFGV, precision);
  if (rc != PD_OK) std::fprintf(stderr, "run_timeloop_gpu: [%d] %s\n", rc, pd_global_error());
  MPI_Finalize();
  return rc == PD_OK ? 0 : 1;
}
