// dpm_simulate: drop-in for the reference `dpm_Simulate` command line
// (dpm_Simulate.cc:27-158). Same options, defaults, configuration echo and
// hist.sim output (Geom.cc:167-192); the transport runs on the GPU through
// libdpmx. Two options are added: -s seed (the reference's seed is fixed at
// 123, Random.cc:3) and -P fp64|fp32 (plain FP64 form or event-based FP32 form).
#include <getopt.h>

#include <cstdio>
#include <cstdlib>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "dpmx.h"

namespace {

std::string gPrimaryParticle("e-");
std::string gInputDataDir("./data");
std::string gOutputFileName("hist.sim");
double gPrimaryEnergy = 15.0;
double gVoxelSize = 1.0;
int gNumPrimaries = 100000;
int gConfigIndex = 0;
unsigned long long gSeed = 123;
std::string gPrecision("fp64");

struct option options[] = {
    {"primary-particle    (possible particle names: e-, gamma)            - default: e-", required_argument, 0, 'p'},
    {"primary-energy      (in [MeV] units)                                - default: 15", required_argument, 0, 'e'},
    {"number-of-histories (number of primary events to simulate)          - default: 1.0E+5", required_argument, 0, 'n'},
    {"input-data-dir      (where the pre-generated data are located)      - default: ./data", required_argument, 0, 'd'},
    {"voxel-size          (size of the voxel/box in [mm])                 - default: 1.0", required_argument, 0, 'b'},
    {"configuration-index (one of the pre-defined configuration index)    - default: 0", required_argument, 0, 'c'},
    {"output-filename     (the filename of the result)                    - default: hist.sim", required_argument, 0, 'o'},
    {"seed                (random seed)                                   - default: 123", required_argument, 0, 's'},
    {"precision           (fp64: plain FP64 form, fp32: event FP32 form)  - default: fp64", required_argument, 0, 'P'},
    {"help", no_argument, 0, 'h'},
    {0, 0, 0, 0}};

void Help() {
  std::cout << "\n " << std::setw(120) << std::setfill('=') << "" << std::setfill(' ') << std::endl;
  std::cout << "  The dpm++ simulation phase (GB300)." << std::endl;
  std::cout << "\n  Usage: dpm_simulate [OPTIONS] \n" << std::endl;
  for (int i = 0; options[i].name != NULL; i++) printf("\t-%c  --%s\n", options[i].val, options[i].name);
  std::cout << "\n " << std::setw(120) << std::setfill('=') << "" << std::setfill(' ') << std::endl;
}

void GetOpt(int argc, char* argv[]) {
  while (true) {
    int optidx = 0;
    int c = getopt_long(argc, argv, "hp:e:n:d:b:c:o:s:P:", options, &optidx);
    if (c == -1) break;
    switch (c) {
      case 'p':
        gPrimaryParticle = optarg;
        if (!(gPrimaryParticle == "e-" || gPrimaryParticle == "gamma")) {
          std::cout << " *** Unknown primary particle name -p: " << optarg << std::endl;
          Help();
          exit(-1);
        }
        break;
      case 'o': gOutputFileName = optarg; break;
      case 'e': gPrimaryEnergy = std::stod(optarg); break;
      case 'n': gNumPrimaries = std::stoi(optarg); break;   // like the reference: "1e5" reads as 1
      case 'd': gInputDataDir = optarg; break;
      case 'b': gVoxelSize = std::stod(optarg); break;
      case 'c': gConfigIndex = std::stoi(optarg); break;
      case 's': gSeed = std::stoull(optarg); break;
      case 'P':
        gPrecision = optarg;
        if (!(gPrecision == "fp64" || gPrecision == "fp32")) {
          std::cout << " *** Unknown precision -P: " << optarg << std::endl;
          Help();
          exit(-1);
        }
        break;
      case 'h': Help(); exit(-1);
      default:
        printf(" *** Unknown input argument: %c\n", c);
        Help();
        exit(-1);
    }
  }
  std::cout << "\n === The dpm++ simulation confguration: \n"
            << "\n     - input data directory  : " << gInputDataDir
            << "\n     - output filename  : " << gOutputFileName
            << "\n     - primary particle      : " << gPrimaryParticle
            << "\n     - primary energy        : " << gPrimaryEnergy << " [MeV]"
            << "\n     - number of histories   : " << gNumPrimaries
            << "\n     - geometry voxel size   : " << gVoxelSize << " [mm]"
            << "\n     - confoguration index   : " << gConfigIndex
            << "\n     - random seed           : " << gSeed
            << "\n     - precision             : " << gPrecision << std::endl;
}

// the geometry index of the reference's pre-defined configurations
// (Configuration.hh:69-111): 1, 2, 3 use slab geometries 1, 2, 3; others 0
int GeomIndex(int config) { return (config >= 1 && config <= 3) ? config : 0; }

}  // namespace

int main(int argc, char* argv[]) {
  GetOpt(argc, argv);
  dpmx_tables* t = nullptr;
  int rc = dpmx_tables_load(gInputDataDir.c_str(), &t);
  if (rc != DPMX_OK) {
    std::cerr << " *** ERROR: " << dpmx_last_error() << std::endl;
    return EXIT_FAILURE;
  }
  const int geom = GeomIndex(gConfigIndex);
  const int cap = 4096;
  std::vector<double> edep(cap, 0.0), steps(cap, 0.0);
  int len = 0;
  std::cout << "\n === Start simulation of N = " << gNumPrimaries << " events === \n" << std::endl;
  rc = dpmx_simulate(t, gNumPrimaries, gPrimaryEnergy, gPrimaryParticle == "e-" ? 1 : 0, gVoxelSize, geom, gSeed,
                     gPrecision == "fp64" ? DPMX_FP64_PLAIN : DPMX_FP32_EVENT, edep.data(), steps.data(), cap, &len);
  if (rc != DPMX_OK) {
    std::cerr << " *** ERROR in the simulation: " << dpmx_last_error() << std::endl;
    dpmx_tables_free(t);
    return EXIT_FAILURE;
  }
  std::cout << "\n === End simulation of N = " << gNumPrimaries << " events === \n" << std::endl;
  if (len > cap) len = cap;
  rc = dpmx_write_hist(t, gOutputFileName.c_str(), geom, gVoxelSize, gNumPrimaries, edep.data(), steps.data(), len);
  if (rc != DPMX_OK) {
    std::cerr << " *** ERROR in Geom::Write(): " << dpmx_last_error() << std::endl;
  } else {
    std::cout << " === Energy deposit histogram is written to the file:  " << gOutputFileName << "\n" << std::endl;
  }
  dpmx_tables_free(t);
  return 0;
}
