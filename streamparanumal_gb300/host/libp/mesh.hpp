// mesh_t of the GB300 drop-in: the structured hex box of the reference's
// mesh_t::Setup (libs/mesh/meshSetup.cpp:31-82) at one rank, reduced to what the
// BS6-BS8 drivers use -- degree, node counts, global ids and the ogs handle
// (ogs.Setup(Signed, Auto, unique=true), libs/mesh/meshGatherScatterSetup.cpp:31-44).
#pragma once

#include "ogs.hpp"

namespace libp {

void meshAddSettings(settings_t& settings);
void meshReportSettings(settings_t& settings);

class mesh_t {
 public:
  platform_t platform;
  settings_t settings;
  comm_t comm;
  int rank = 0, size = 1;

  int N = 0, Nq = 0, Np = 0;  // degree, nodes per edge, nodes per element
  dlong Nelements = 0;
  hlong NelementsGlobal = 0;
  int nx = 0, ny = 0, nz = 0;
  unsigned long long permSeed = 0;  // element-slot permutation (0 = lexicographic)

  memory<hlong> globalIds;
  ogs::ogs_t ogs;

  mesh_t() = default;
  mesh_t(platform_t& _platform, settings_t& _settings, comm_t _comm) {
    Setup(_platform, _settings, _comm);
  }
  void Setup(platform_t& _platform, settings_t& _settings, comm_t _comm);
};

}  // namespace libp
