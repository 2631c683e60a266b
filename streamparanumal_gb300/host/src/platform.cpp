// platform_t of the GB300 drop-in: CUDA device and stream, and the binding of the
// reference's BS kernel names to libspgb300 entry points.
#include <cstring>
#include <map>
#include <mutex>

#include "platform.hpp"

namespace libp {

void checkStatus(sp_status st, const char* what) {
  LIBP_ABORT(what << ": " << sp_status_string(st) << ": " << sp_last_error_string(),
             st != SP_SUCCESS);
}

void platformAddSettings(settings_t& settings) {
  // libs/core/platformSettings.cpp:31-48; this build runs the CUDA mode only
  settings.newSetting("-m", "--mode", "THREAD MODEL", "CUDA",
                      "OCCA's Parallel execution platform", {"Serial", "OpenMP", "CUDA", "HIP",
                                                             "OpenCL"});
  settings.newSetting("-pl", "--platform", "PLATFORM NUMBER", "0",
                      "Parallel platform number (used in OpenCL mode)");
  settings.newSetting("-d", "--device", "DEVICE NUMBER", "0", "Parallel device number");
}

void platformReportSettings(settings_t& settings) {
  std::printf("Platform Settings:\n\n");
  settings.reportSetting("THREAD MODEL");
  settings.reportSetting("DEVICE NUMBER");
}

platform_t::platform_t(settings_t& settings) : st_(std::make_shared<state>()) {
  st_->settings = &settings;
  comm = settings.comm;
  LIBP_ABORT("This build runs the CUDA mode only (THREAD MODEL = CUDA)",
             !settings.compareSetting("THREAD MODEL", "CUDA"));
  settings.getSetting("DEVICE NUMBER", st_->device);
  int ndev = 0;
  LIBP_CUDA_CHECK(cudaGetDeviceCount(&ndev));
  LIBP_ABORT("DEVICE NUMBER " << st_->device << " but " << ndev << " devices",
             st_->device < 0 || st_->device >= ndev);
  LIBP_CUDA_CHECK(cudaSetDevice(st_->device));
  LIBP_CUDA_CHECK(cudaStreamCreateWithFlags(&st_->stream, cudaStreamNonBlocking));
  device = device_t(&st_->stream);
  st_->props["defines/dfloat"] = "double";
  st_->props["defines/dlong"] = "int";
}

namespace {

using Args = std::vector<kernelArg>;

void expect(const Args& a, const char* name, std::initializer_list<kernelArg::Kind> kinds) {
  LIBP_ABORT("kernel " << name << " expects " << kinds.size() << " arguments, got " << a.size(),
             a.size() != kinds.size());
  size_t i = 0;
  for (auto k : kinds) {
    LIBP_ABORT("kernel " << name << ": argument " << i << " has the wrong kind", a[i].kind != k);
    ++i;
  }
}

constexpr auto I = kernelArg::Int;
constexpr auto R = kernelArg::Real;
constexpr auto P = kernelArg::Ptr;

// bs0.okl:27-39: (N, a, b)
sp_status k_bs0(const Args& a, int, cudaStream_t s) {
  expect(a, "bs0", {I, P, P});
  return sp_bs0((int32_t)a[0].i, (const double*)a[1].p, (double*)a[2].p, (sp_stream_t)s);
}
// bs1.okl:27-34: (N, a, b)
sp_status k_bs1(const Args& a, int, cudaStream_t s) {
  expect(a, "bs1", {I, P, P});
  return sp_bs1_copy_f64(a[0].i, (const double*)a[1].p, (double*)a[2].p, (sp_stream_t)s);
}
// bs2.okl:27-36: (N, alpha, x, beta, y)
sp_status k_bs2(const Args& a, int, cudaStream_t s) {
  expect(a, "bs2", {I, R, P, R, P});
  return sp_bs2_axpy_f64(a[0].i, a[1].d, (const double*)a[2].p, a[3].d, (double*)a[4].p,
                         (sp_stream_t)s);
}
// Scratch of the single-launch reductions, one per device: allocated and zeroed on
// the first call that needs it (a driver's warm-up calls come before its timed
// loop) and kept until exit, as the reference keeps its kernel objects
// (libs/ogs/ogsUtils.cpp:39-43).  Every bound kernel runs on the platform's one
// stream, so calls sharing it never overlap.
void* reduce_scratch() {
  static std::mutex mu;
  static std::map<int, void*> bufs;
  int dev = 0;
  LIBP_CUDA_CHECK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  void*& p = bufs[dev];
  if (!p) {
    LIBP_CUDA_CHECK(cudaMalloc(&p, sp_reduce_scratch_bytes()));
    LIBP_CUDA_CHECK(cudaMemset(p, 0, sp_reduce_scratch_bytes()));
  }
  return p;
}

// bs3.okl:27-64: (Nblocks, N, a, norm).  The integer-pipe norm by default (the
// result lands in norm[0], norm[1..Nblocks) = 0, so bs3_2 returns it); the
// order-exact kernel under the knob reduce.norm_exact = 1.
sp_status k_bs3_1(const Args& a, int bs, cudaStream_t s) {
  expect(a, "bs3_1", {I, I, P, P});
  int64_t exact = 0;
  if (sp_status st = sp_tune_get("reduce.norm_exact", &exact)) return st;
  if (exact)
    return sp_bs3_1_f64(bs, (int32_t)a[0].i, a[1].i, (const double*)a[2].p, (double*)a[3].p,
                        (sp_stream_t)s);
  return sp_bs3_1_fast_f64(bs, (int32_t)a[0].i, a[1].i, (const double*)a[2].p, (double*)a[3].p,
                           reduce_scratch(), (sp_stream_t)s);
}
// bs4.okl:27-65: (Nblocks, N, a, b, ddot)
sp_status k_bs4_1(const Args& a, int bs, cudaStream_t s) {
  expect(a, "bs4_1", {I, I, P, P, P});
  return sp_bs4_1_f64(bs, (int32_t)a[0].i, a[1].i, (const double*)a[2].p, (const double*)a[3].p,
                      (double*)a[4].p, (sp_stream_t)s);
}
// bs5.okl:27-67: (Nblocks, N, Ap, alpha, r, rdotr).  r updated as the reference
// does; r.r on the integer pipe by default (rdotr[0], rdotr[1..Nblocks) = 0, so
// bs5_2 returns it); the order-exact kernel under the knob reduce.rdotr_exact = 1.
sp_status k_bs5_1(const Args& a, int bs, cudaStream_t s) {
  expect(a, "bs5_1", {I, I, P, R, P, P});
  int64_t exact = 0;
  if (sp_status st = sp_tune_get("reduce.rdotr_exact", &exact)) return st;
  if (exact)
    return sp_bs5_1_f64(bs, (int32_t)a[0].i, a[1].i, (const double*)a[2].p, a[3].d,
                        (double*)a[4].p, (double*)a[5].p, (sp_stream_t)s);
  return sp_bs5_1_fast_f64(bs, (int32_t)a[0].i, a[1].i, (const double*)a[2].p, a[3].d,
                           (double*)a[4].p, (double*)a[5].p, reduce_scratch(), (sp_stream_t)s);
}
// bs3_2 / bs4_2 / bs5_2 (identical): (Nblocks, a, out)
sp_status k_finish(const Args& a, int bs, cudaStream_t s) {
  expect(a, "bs*_2", {I, P, P});
  return sp_reduce_finish_f64(bs, (int32_t)a[0].i, (const double*)a[1].p, (double*)a[2].p,
                              (sp_stream_t)s);
}

struct binding {
  const char* name;
  kernel_t::fn_t fn;
};
const binding kBindings[] = {
    {"bs0", k_bs0},       {"bs1", k_bs1},       {"bs2", k_bs2},       {"bs3_1", k_bs3_1},
    {"bs3_2", k_finish},  {"bs4_1", k_bs4_1},   {"bs4_2", k_finish},  {"bs5_1", k_bs5_1},
    {"bs5_2", k_finish},
};

}  // namespace

kernel_t platform_t::buildKernel(const std::string& fileName, const std::string& kernelName,
                                 properties_t& kernelInfo) {
  LIBP_ABORT("Platform not initialized.", !st_);
  int bs = 256;
  if (kernelInfo.has("defines/p_blockSize")) bs = std::stoi(kernelInfo.get("defines/p_blockSize"));
  for (const binding& b : kBindings)
    if (kernelName == b.name) return kernel_t(kernelName, b.fn, bs, st_->stream);
  LIBP_FORCE_ABORT("No GB300 kernel bound to " << kernelName << " (" << fileName << ")");
}

timePoint_t PlatformTime(platform_t& platform) {
  platform.finish();
  return Time();
}

timePoint_t GlobalPlatformTime(platform_t& platform) {
  platform.finish();
  platform.comm.Barrier();
  return Time();
}

}  // namespace libp
