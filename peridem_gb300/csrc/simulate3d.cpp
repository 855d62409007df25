// simulate3d.cpp -- drop-in for PeriDEM's run/simulate3d.cpp: same command line
// (`-c <main.conf> -i <setup.h5> -o <output dir>`, defaults config/main.conf, data/hdf5/all.h5,
// output/hdf5/), same config grammar, setup schema and output files, with the time loop on the
// GPU. Extra option: `-p fp32c` selects the FP32-compensated form (default fp64, bit-exact).
#include <unistd.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <string>

#include "peridem_gb300.h"

extern "C" const char *pd_files_error(void);

int main(int argc, char *argv[]) {
  std::string conf = "config/main.conf", setup = "data/hdf5/all.h5", outdir = "output/hdf5/";
  int precision = PD_FP64;
  int opt;
  while ((opt = getopt(argc, argv, "c:i:o:p:")) != -1) {
    switch (opt) {
      case 'c': conf = optarg; break;
      case 'i': setup = optarg; break;
      case 'o': outdir = optarg; break;
      case 'p':
        if (std::strcmp(optarg, "fp32c") == 0) precision = PD_FP32C;
        else if (std::strcmp(optarg, "fp64") == 0) precision = PD_FP64;
        else {
          std::cerr << "unknown precision form " << optarg << " (fp64 | fp32c)\n";
          return 2;
        }
        break;
      case ':': std::printf("option needs a value\n"); break;
      default: break;
    }
  }
  std::cout << "GPU processes 1" << std::endl;
  std::cout << "Reading input setup file: " << setup << std::endl;
  auto start = std::chrono::system_clock::now();
  pd_sim *sim = nullptr;
  int rc = pd_open(conf.c_str(), setup.c_str(), outdir.c_str(), precision, &sim);
  if (rc != PD_OK) {
    std::cerr << "Error: " << pd_files_error() << " " << pd_global_error() << std::endl;
    return 1;
  }
  rc = pd_run(sim);
  if (rc != PD_OK) {
    std::cerr << "Error: " << pd_last_error(sim) << " " << pd_files_error() << std::endl;
    pd_close(sim);
    return 1;
  }
  pd_close(sim);
  auto stop = std::chrono::system_clock::now();
  std::cout << "Runtime: " << std::chrono::duration_cast<std::chrono::seconds>(stop - start).count() << "s"
            << std::endl;
  return 0;
}
