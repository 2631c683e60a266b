// One executable for the nine drivers, installed as BS0 ... BS8; the program name
// selects the benchmark (as the reference's separate BSx executables do).  The
// command line of each is the reference's (BS/BSx/src/bsxSettings.cpp).
#include <cstring>
#include <iostream>
#include <string>

#include "bs.hpp"

using namespace libp;

int main(int argc, char** argv) {
  std::string prog = argv[0];
  const size_t slash = prog.find_last_of('/');
  if (slash != std::string::npos) prog = prog.substr(slash + 1);
  int which = -1;
  if (prog.size() == 3 && prog[0] == 'B' && prog[1] == 'S' && prog[2] >= '0' && prog[2] <= '8')
    which = prog[2] - '0';
  if (which < 0 && argc > 1 && std::strlen(argv[1]) == 3 && argv[1][0] == 'B' &&
      argv[1][1] == 'S' && argv[1][2] >= '0' && argv[1][2] <= '8') {
    which = argv[1][2] - '0';
    ++argv;
    --argc;
  }
  if (which < 0) {
    std::cerr << "usage: BS0..BS8 [options]  (or " << prog << " BSx [options])\n";
    return 2;
  }
  try {
    Comm::Init(argc, argv);
    comm_t comm(Comm::World().Dup());
    settings_t settings(comm);
    if (which == 0) bs0Settings(settings);
    else if (which <= 5) bsVecSettings(settings);
    else bsOgsSettings(settings);
    settings.parseSettings(argc, argv);
    if (settings.compareSetting("VERBOSE", "TRUE")) settings.report();
    platform_t platform(settings);
    if (which == 0) {
      bs0Run(platform, settings);
    } else if (which <= 5) {
      bsVecRun(which, platform, settings);
    } else {
      bsOgsApplyTuning(settings);
      mesh_t mesh(platform, settings, comm);
      bsOgsRun(which, platform, settings, mesh);
    }
    Comm::Finalize();
  } catch (const libp::exception& e) {
    std::cerr << e.what();
    return 1;
  }
  return LIBP_SUCCESS;
}
