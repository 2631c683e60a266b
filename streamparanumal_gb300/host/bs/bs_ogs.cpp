// BS6 gather, BS7 scatter and BS8 gather+scatter drivers of the GB300 drop-in: the
// timing loops and output rows of the reference's BS/BS{6,7,8}/src/bs*Run.cpp, with
// mesh.ogs served by libspgb300.  Added option: -fp/--precision FP32 runs the
// operators on FP32 node data (byte accounting with 4-byte values).
#include "bs.hpp"

namespace libp {

void bsOgsSettings(settings_t& s) {
  platformAddSettings(s);
  meshAddSettings(s);
  s.newSetting("-fp", "--precision", "PRECISION", "FP64", "Storage precision", {"FP64", "FP32"});
  s.newSetting("-v", "--verbose", "VERBOSE", "FALSE", "Enable verbose output", {"TRUE", "FALSE"});
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
