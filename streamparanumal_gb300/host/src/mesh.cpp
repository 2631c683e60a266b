// mesh_t of the GB300 drop-in: structured hex box ids and the ogs handle.
#include "mesh.hpp"

namespace libp {

void meshAddSettings(settings_t& settings) {
  // libs/mesh/meshSettings.cpp:27-50, plus the element-slot permutation seed
  settings.newSetting("-e", "--elements", "ELEMENT TYPE", "Hex", "Type of mesh elements",
                      {"Tri", "Quad", "Tet", "Hex"});
  settings.newSetting("-nx", "--dimx", "BOX NX", "50", "Number of elements in X-dimension per rank");
  settings.newSetting("-ny", "--dimy", "BOX NY", "50", "Number of elements in Y-dimension per rank");
  settings.newSetting("-nz", "--dimz", "BOX NZ", "50", "Number of elements in Z-dimension per rank");
  settings.newSetting("-p", "--degree", "POLYNOMIAL DEGREE", "3",
                      "Degree of polynomial finite element space",
                      {"1", "2", "3", "4", "5", "6", "7", "8", "9", "10", "11", "12", "13", "14",
                       "15"});
  settings.newSetting("-ps", "--perm-seed", "PERMUTATION SEED", "0",
                      "Seed of a random permutation of the element slots (0: lexicographic)");
}

void meshReportSettings(settings_t& settings) {
  settings.reportSetting("ELEMENT TYPE");
  settings.reportSetting("BOX NX");
  settings.reportSetting("BOX NY");
  settings.reportSetting("BOX NZ");
  settings.reportSetting("POLYNOMIAL DEGREE");
  settings.reportSetting("PERMUTATION SEED");
}

void mesh_t::Setup(platform_t& _platform, settings_t& _settings, comm_t _comm) {
  platform = _platform;
  settings = _settings;
  comm = _comm.Dup();
  rank = comm.rank();
  size = comm.size();
  LIBP_ABORT("This build's mesh_t supports hexahedral boxes only (-e Hex)",
             !settings.compareSetting("ELEMENT TYPE", "Hex"));
  settings.getSetting("POLYNOMIAL DEGREE", N);
  settings.getSetting("BOX NX", nx);
  settings.getSetting("BOX NY", ny);
  settings.getSetting("BOX NZ", nz);
  if (settings.hasSetting("PERMUTATION SEED")) settings.getSetting("PERMUTATION SEED", permSeed);
  Nq = N + 1;
  Np = Nq * Nq * Nq;
  Nelements = nx * ny * nz;
  NelementsGlobal = Nelements;
  const long long Nlocal = (long long)Nelements * Np;
  LIBP_ABORT("Local node count " << Nlocal << " exceeds dlong", Nlocal > 2147483647LL);
  // global ids generated and grouped on the device; the signed ids (one positive
  // member per group) are then kept on the host as mesh_t::globalIds
  deviceMemory<hlong> o_globalIds = platform.malloc<hlong>((size_t)Nlocal);
  checkStatus(sp_mesh_box_hex_ids_device(nx, ny, nz, N, permSeed,
                                         reinterpret_cast<int64_t*>(o_globalIds.ptr()),
                                         (sp_stream_t)platform.stream()),
              "mesh_t::Setup");
  const bool verbose = settings.hasSetting("VERBOSE") && settings.compareSetting("VERBOSE", "TRUE");
  ogs.Setup((dlong)Nlocal, o_globalIds, comm, ogs::Signed, ogs::Auto, /*unique=*/true, verbose,
            platform);
  globalIds.malloc((size_t)Nlocal);
  o_globalIds.copyTo(globalIds);
}

}  // namespace libp
