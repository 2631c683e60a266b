// BS6 gather, BS7 scatter and BS8 gather+scatter drivers of the GB300 drop-in: the
// timing loops and output rows of the reference's BS/BS{6,7,8}/src/bs*Run.cpp, with
// mesh.ogs served by libspgb300.  Added option: -fp/--precision FP32 runs the
// operators on FP32 node data (byte accounting with 4-byte values).
#include "bs.hpp"

#include <unistd.h>

#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>

namespace libp {

void bsOgsSettings(settings_t& s) {
  platformAddSettings(s);
  meshAddSettings(s);
  s.newSetting("-fp", "--precision", "PRECISION", "FP64", "Storage precision", {"FP64", "FP32"});
  s.newSetting("-v", "--verbose", "VERBOSE", "FALSE", "Enable verbose output", {"TRUE", "FALSE"});
  s.newSetting("-t", "--tuning", "TUNING FILE", "DEFAULT",
               "Per-degree kernel table (DEFAULT: the package's, NONE: library defaults)");
}

// The table's text form holds one line per degree and layout:
//   p7_perm ogs.order=1 ogs.rows=1 ogs.kernel=2 ...
// The line for this run's degree (and permuted layout, else the plain one) is
// applied through sp_tune_set.
void bsOgsApplyTuning(settings_t& s) {
  std::string file;
  s.getSetting("TUNING FILE", file);
  if (file == "NONE") return;
  if (file == "DEFAULT") {
    char exe[4096];
    const ssize_t len = readlink("/proc/self/exe", exe, sizeof(exe) - 1);
    if (len <= 0) return;
    exe[len] = 0;
    std::string dir(exe);
    dir = dir.substr(0, dir.find_last_of('/'));          // .../bin
    file = dir.substr(0, dir.find_last_of('/')) + "/tuning/gb300.txt";
  }
  std::ifstream in(file);
  if (!in) {
    LIBP_ABORT("Cannot read tuning file " << file, !s.compareSetting("TUNING FILE", "DEFAULT"));
    return;
  }
  int p = 0;
  long long seed = 0;
  s.getSetting("POLYNOMIAL DEGREE", p);
  if (s.hasSetting("PERMUTATION SEED")) s.getSetting("PERMUTATION SEED", seed);
  const std::string want = "p" + std::to_string(p), wantPerm = want + "_perm";
  std::string line, plain, perm;
  while (std::getline(in, line)) {
    const std::string key = line.substr(0, line.find(' '));
    if (key == want) plain = line;
    if (key == wantPerm) perm = line;
  }
  const std::string& use = (seed != 0 && !perm.empty()) ? perm : plain;
  std::istringstream fields(use);
  std::string field;
  fields >> field;  // the key
  while (fields >> field) {
    const size_t eq = field.find('=');
    if (eq == std::string::npos) continue;
    const std::string knob = field.substr(0, eq);
    const long long value = std::stoll(field.substr(eq + 1));
    checkStatus(sp_tune_set(knob.c_str(), value), "tuning file");
  }
  if (s.compareSetting("VERBOSE", "TRUE") && !use.empty())
    std::printf("tuning: %s\n", use.c_str());
}

namespace {

template <typename T>
void run(int which, platform_t& platform, mesh_t& mesh) {
  const dlong N = mesh.Np * mesh.Nelements;
  const dlong Ngather = mesh.ogs.Ngather;
  deviceMemory<T> o_q = platform.malloc<T>(N);
  deviceMemory<T> o_gq = platform.malloc<T>(Ngather > 0 ? Ngather : 1);
  auto op = [&]() {
    if (which == 6) mesh.ogs.Gather(o_gq, o_q, 1, ogs::Add, ogs::Trans);   // bs6Run.cpp:47
    else if (which == 7) mesh.ogs.Scatter(o_q, o_gq, 1, ogs::NoTrans);     // bs7Run.cpp:47
    else mesh.ogs.GatherScatter(o_q, 1, ogs::Add, ogs::Sym);               // bs8Run.cpp:45
  };
  for (int n = 0; n < 5; ++n) op();  // warm-up
  const int Ntests = (which == 8) ? 50 : 20;
  timePoint_t start = GlobalPlatformTime(platform);
  for (int n = 0; n < Ntests; ++n) op();
  timePoint_t end = GlobalPlatformTime(platform);
  const double elapsedTime = ElapsedTime(start, end) / Ntests;

  hlong NtotalGlobal = (hlong)mesh.Nelements * mesh.Np;
  mesh.comm.Allreduce(NtotalGlobal);
  const hlong NgatherGlobal = mesh.ogs.NgatherGlobal;
  // byte accounting: bs6Run.cpp:58-63, bs7Run.cpp:58-63, bs8Run.cpp:56-61
  size_t bytesIn = (NgatherGlobal + 1) * sizeof(dlong) + NtotalGlobal * sizeof(dlong);
  size_t bytesOut = 0;
  double flops = 0;
  const char* title = "";
  if (which == 6) {
    bytesIn += NtotalGlobal * sizeof(T);
    bytesOut += NgatherGlobal * sizeof(T);
    flops = (double)NtotalGlobal;
    title = "Gather";
  } else if (which == 7) {
    bytesIn += NgatherGlobal * sizeof(T);
    bytesOut += NtotalGlobal * sizeof(T);
    title = "Scatter";
  } else {
    bytesIn += NtotalGlobal * sizeof(T);
    bytesOut += NtotalGlobal * sizeof(T);
    flops = (double)NtotalGlobal;
    title = "GatherScatter";
  }
  const size_t bytes = bytesIn + bytesOut;
  const hlong Ndofs = NgatherGlobal;
  if (mesh.rank == 0)
    std::printf("BS%d = [%d, " hlongFormat ", %5.4le, %5.4le, %6.2f, %6.2f]; %% %s [N, DOFs, "
                "elapsed, DOFs/(ranks*s), avg BW (GB/s), avg GFLOPs] \n",
                which, mesh.N, Ndofs, elapsedTime, Ndofs / (mesh.size * elapsedTime),
                bytes / (1.0e9 * elapsedTime), flops / (1.0e9 * elapsedTime), title);
}

}  // namespace

void bsOgsRun(int which, platform_t& platform, settings_t& settings, mesh_t& mesh) {
  if (settings.compareSetting("PRECISION", "FP32")) run<float>(which, platform, mesh);
  else run<dfloat>(which, platform, mesh);
}

}  // namespace libp
