// BS0-BS5 drivers of the GB300 drop-in.  Same command line, same timing loop and
// same output rows as the reference's BS/BS{0..5}/src/bs*Run.cpp; the kernels are
// built by platform_t::buildKernel and run through libspgb300.
// Added option: -fp/--precision FP32 runs the FP32-storage forms (BS1 copy, BS2
// axpy, BS3 norm and BS4 dot with compensated FP32 lanes, BS5's r += alpha Ap and
// r.r in one launch); -cg/--cg-full TRUE runs BS5 as the full CG update
// x += alpha p, r -= alpha Ap, r.r (FP64 or FP32 storage).
#include <string>

#include "bs.hpp"

namespace libp {

void bs0Settings(settings_t& s) {
  platformAddSettings(s);
  s.newSetting("-n", "--Nlaunch", "NLAUNCHES", "0", "Number of small kernels to launch");
  s.newSetting("-nmin", "--NlaunchMin", "NLAUNCHMIN", "0",
               "Minimum number of small kernels to launch");
  s.newSetting("-nmax", "--NlaunchMax", "NLAUNCHMAX", "0",
               "Maximum number of small kernels to launch");
  s.newSetting("-s", "--step", "NLAUNCHSTEP", "1", "Step size of small kernels to launch");
  s.newSetting("-g", "--graph", "GRAPH", "FALSE",
               "Replay the launches from one captured CUDA graph", {"TRUE", "FALSE"});
  s.newSetting("-v", "--verbose", "VERBOSE", "FALSE", "Enable verbose output", {"TRUE", "FALSE"});
}

void bsVecSettings(settings_t& s) {
  platformAddSettings(s);
  s.newSetting("-b", "--bytes", "BYTES", "0", "Array size in bytes");
  s.newSetting("-bmin", "--bmin", "BMIN", "0", "Minimum array size in bytes");
  s.newSetting("-bmax", "--bmax", "BMAX", "0", "Maximum array size in bytes");
  s.newSetting("-s", "--bstep", "BSTEP", "1048576", "Array step size in bytes");
  s.newSetting("-fp", "--precision", "PRECISION", "FP64", "Storage precision", {"FP64", "FP32"});
  s.newSetting("-cg", "--cg-full", "CG FULL", "FALSE",
               "BS5 as the full CG update x+=alpha p, r-=alpha Ap, r.r", {"TRUE", "FALSE"});
  s.newSetting("-ex", "--exact-norm", "EXACT NORM", "FALSE",
               "BS3 norm and BS5 r.r in the reference's summation order (bit-identical; "
               "bound by the FP64 pipe) instead of on the integer pipe", {"TRUE", "FALSE"});
  s.newSetting("-v", "--verbose", "VERBOSE", "FALSE", "Enable verbose output", {"TRUE", "FALSE"});
}

// bs0Run.cpp:30-82
void bs0Run(platform_t& platform, settings_t& settings) {
  properties_t kernelInfo = platform.props();
  kernelInfo["defines/p_blockSize"] = "1";
  kernel_t kernel = platform.buildKernel("BS/BS0/okl/bs0.okl", "bs0", kernelInfo);

  int Nlaunches = 10, NlaunchMin = 1, NlaunchMax = 1024, NlaunchStep = 1;
  settings.getSetting("NLAUNCHES", Nlaunches);
  settings.getSetting("NLAUNCHMIN", NlaunchMin);
  settings.getSetting("NLAUNCHMAX", NlaunchMax);
  settings.getSetting("NLAUNCHSTEP", NlaunchStep);
  if (!(Nlaunches | NlaunchMin | NlaunchMax)) Nlaunches = 10;
  const bool graph = settings.compareSetting("GRAPH", "TRUE");

  const int N = 1;
  deviceMemory<dfloat> o_a = platform.malloc<dfloat>(N);
  deviceMemory<dfloat> o_b = platform.malloc<dfloat>(N);
  for (int w = 0; w < 100; ++w) kernel(N, o_a, o_b);

  if (Nlaunches) {
    NlaunchMin = NlaunchMax = Nlaunches;
    std::printf("BS0 = [");
  } else {
    std::printf("%%Launch Latency [Nlaunches, time per launch, elapsed]\n");
    std::printf("BS0 = [\n");
  }
  for (Nlaunches = NlaunchMin; Nlaunches <= NlaunchMax; Nlaunches += NlaunchStep) {
    sp_graph* g = nullptr;
    if (graph) {
      checkStatus(sp_bs0_graph_create(Nlaunches, N, o_a.ptr(), o_b.ptr(),
                                      (sp_stream_t)platform.stream(), &g),
                  "sp_bs0_graph_create");
      checkStatus(sp_graph_launch(g, (sp_stream_t)platform.stream()), "sp_graph_launch");
    }
    timePoint_t start = PlatformTime(platform);
    if (graph) {
      checkStatus(sp_graph_launch(g, (sp_stream_t)platform.stream()), "sp_graph_launch");
    } else {
      for (int n = 0; n < Nlaunches; ++n) kernel(N, o_a, o_b);
    }
    timePoint_t end = PlatformTime(platform);
    if (g) sp_graph_destroy(g);
    const double elapsed = ElapsedTime(start, end);
    std::printf("%d %5.4e %5.4e", Nlaunches, elapsed / Nlaunches, elapsed);
    if (Nlaunches < NlaunchMax) std::printf(";\n");
  }
  std::printf("]; %%Launch Latency [Nlaunches, time per launch, elapsed]\n");
}

namespace {

struct sweep_t {
  size_t Nmin = 0, Nmax = 0, Nstep = 1;
  bool single = false;
};

// The byte-range logic shared by bs1Run.cpp:31-67 ... bs5Run.cpp:31-76.
sweep_t sweep(settings_t& settings, size_t sc) {
  size_t B = 0, Bmin = 0, Bmax = 0, Bstep = 0;
  settings.getSetting("BYTES", B);
  settings.getSetting("BMIN", Bmin);
  settings.getSetting("BMAX", Bmax);
  settings.getSetting("BSTEP", Bstep);
  if (!(B | Bmin | Bmax)) B = 1073741824;
  if (B) Bmax = B;
  sweep_t s;
  s.Nmin = Bmin / sc;
  s.Nmax = Bmax / sc;
  s.Nstep = (Bstep / sc > 0) ? Bstep / sc : 1;
  if (B) {
    s.single = true;
    s.Nmin = s.Nmax = B / sc;
  }
  return s;
}

void open_row(int bs, const sweep_t& s, const char* title) {
  if (s.single) {
    std::printf("BS%d = [", bs);
  } else {
    std::printf("%%%s [DOFs, elapsed, DOFs/s, BW (GB/s)]\n", title);
    std::printf("BS%d = [\n", bs);
  }
}

void print_entry(size_t N, double elapsed, size_t bytes, size_t Nmax) {
  std::printf("%d %5.4e %5.4e %6.2f", (int)N, elapsed, N / elapsed,
              (double)(bytes / 1.e9) / elapsed);
  if (N < Nmax) std::printf(";\n");
}

int nblock_for(size_t N, int blockSize) {
  int nb = (int)((N + blockSize - 1) / blockSize);
  return nb > blockSize ? blockSize : (nb < 1 ? 1 : nb);
}

}  // namespace

// BS1 copy (bs1Run.cpp:29-91), BS2 axpy (bs2Run.cpp:29-94), BS3 norm (bs3Run.cpp:29-99),
// BS4 dot (bs4Run.cpp:29-99), BS5 CG update (bs5Run.cpp:29-103).
void bsVecRun(int which, platform_t& platform, settings_t& settings) {
  const bool fp32 = settings.compareSetting("PRECISION", "FP32");
  const bool cgFull = (which == 5) && settings.compareSetting("CG FULL", "TRUE");
  if (which == 3 || which == 5)
    checkStatus(sp_tune_set(which == 3 ? "reduce.norm_exact" : "reduce.rdotr_exact",
                            settings.compareSetting("EXACT NORM", "TRUE") ? 1 : 0),
                "EXACT NORM");
  const size_t word = fp32 ? sizeof(float) : sizeof(dfloat);
  // entries moved per DOF by each benchmark (the reference's `sc` / word size)
  const size_t perEntry[6] = {0, 2, 3, 1, 2, cgFull ? 6 : 3};
  const char* titles[6] = {"", "Copy", "AXPY", "Norm", "Dot", "CG Update"};
  const size_t sc = perEntry[which] * word;
  const sweep_t sw = sweep(settings, sc);
  const int blockSize = (which == 5) ? 1024 : 256;  // bs5Setup.cpp:37 (CUDA mode)

  properties_t kernelInfo = platform.props();
  kernelInfo["defines/p_blockSize"] = std::to_string(blockSize);
  kernel_t kernel1, kernel2;
  const std::string okl = "BS/BS" + std::to_string(which) + "/okl/bs" + std::to_string(which) +
                          ".okl";
  if (!fp32 && !cgFull) {
    if (which <= 2) {
      kernel1 = platform.buildKernel(okl, "bs" + std::to_string(which), kernelInfo);
    } else {
      kernel1 = platform.buildKernel(okl, "bs" + std::to_string(which) + "_1", kernelInfo);
      kernel2 = platform.buildKernel(okl, "bs" + std::to_string(which) + "_2", kernelInfo);
    }
  }

  const size_t Nmax = sw.Nmax;
  const size_t nvec = (which == 5 && cgFull) ? 4 : 2;
  std::vector<deviceMemory<dfloat>> v64;
  std::vector<deviceMemory<float>> v32;
  for (size_t i = 0; i < nvec; ++i) {
    if (fp32) v32.push_back(platform.malloc<float>(Nmax));
    else v64.push_back(platform.malloc<dfloat>(Nmax));
  }
  deviceMemory<dfloat> o_tmp = platform.malloc<dfloat>(blockSize);
  deviceMemory<dfloat> o_res = platform.malloc<dfloat>(1);
  deviceMemory<char> o_scratch = platform.malloc<char>(sp_reduce_scratch_bytes() + 256);
  LIBP_CUDA_CHECK(cudaMemset(o_scratch.ptr(), 0, o_scratch.size()));
  void* scratch = reinterpret_cast<void*>(
      (reinterpret_cast<uintptr_t>(o_scratch.ptr()) + 255) & ~uintptr_t(255));
  const dfloat alpha = 1.0, beta = 1.0;  // bs2Run.cpp:52-53, bs5Run.cpp:55
  const sp_stream_t s = (sp_stream_t)platform.stream();

  auto call = [&](size_t N) {
    if (fp32) {
      switch (which) {
        case 1: checkStatus(sp_bs1_copy_f32(N, v32[0].ptr(), v32[1].ptr(), s), "BS1"); break;
        case 2:
          checkStatus(sp_bs2_axpy_f32(N, (float)alpha, v32[0].ptr(), (float)beta, v32[1].ptr(), s),
                      "BS2");
          break;
        case 3: checkStatus(sp_norm2_f32(N, v32[0].ptr(), o_res.ptr(), scratch, s), "BS3"); break;
        case 4:
          checkStatus(sp_dot_f32(N, v32[0].ptr(), v32[1].ptr(), o_res.ptr(), scratch, s), "BS4");
          break;
        case 5:
          if (cgFull)
            checkStatus(sp_cg_update_f32(N, alpha, v32[0].ptr(), v32[1].ptr(), v32[2].ptr(),
                                         v32[3].ptr(), o_res.ptr(), scratch, s),
                        "BS5");
          else
            checkStatus(sp_cg_update_ref_f32(N, alpha, v32[0].ptr(), v32[1].ptr(), o_res.ptr(),
                                             scratch, s),
                        "BS5");
          break;
      }
      return;
    }
    if (cgFull) {
      checkStatus(sp_cg_update_f64(N, alpha, v64[0].ptr(), v64[1].ptr(), v64[2].ptr(),
                                   v64[3].ptr(), o_res.ptr(), scratch, s),
                  "BS5");
      return;
    }
    const int Nblock = nblock_for(N, blockSize);
    switch (which) {
      case 1: kernel1((int)N, v64[0], v64[1]); break;                       // b = a
      case 2: kernel1((int)N, alpha, v64[0], beta, v64[1]); break;          // b = alpha*a + beta*b
      case 3: kernel1(Nblock, (int)N, v64[0], o_tmp); kernel2(Nblock, o_tmp, o_res); break;
      case 4: kernel1(Nblock, (int)N, v64[0], v64[1], o_tmp); kernel2(Nblock, o_tmp, o_res); break;
      case 5:
        kernel1(Nblock, (int)N, v64[0], alpha, v64[1], o_tmp);
        kernel2(Nblock, o_tmp, o_res);
        break;
    }
  };

  for (int n = 0; n < 5; ++n) call(Nmax);  // warm-up
  open_row(which, sw, titles[which]);
  for (size_t N = sw.Nmin; N <= sw.Nmax; N += sw.Nstep) {
    timePoint_t start = GlobalPlatformTime(platform);
    const int Ntests = 20;
    for (int n = 0; n < Ntests; ++n) call(N);
    timePoint_t end = GlobalPlatformTime(platform);
    const double elapsed = ElapsedTime(start, end) / Ntests;
    print_entry(N, elapsed, N * sc, sw.Nmax);
    if (N == sw.Nmax) break;
  }
  std::printf("]; %%%s [DOFs, elapsed, DOFs/s, BW (GB/s)]\n", titles[which]);
}

}  // namespace libp
