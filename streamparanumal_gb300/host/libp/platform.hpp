// platform_t, deviceMemory<T> and kernel_t of the GB300 drop-in (the call shapes of
// the reference's include/platform.hpp:60-176 and include/memory.hpp:284-454).
// The OCCA device is replaced by the CUDA runtime for memory and streams and by
// libspgb300.so (include/sp_capi.h) for every kernel.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <string>
#include <type_traits>
#include <vector>

#include "core.hpp"
#include "sp_capi.h"

namespace libp {

// Throws like LIBP_ABORT when a C-ABI call fails.
void checkStatus(sp_status st, const char* what);

#define LIBP_CUDA_CHECK(expr)                                                         \
  do {                                                                                \
    cudaError_t _e = (expr);                                                          \
    LIBP_ABORT(#expr << " failed: " << cudaGetErrorString(_e), _e != cudaSuccess);    \
  } while (0)

// Device buffer with shared ownership and non-owning offset views.
template <typename T>
class deviceMemory {
  std::shared_ptr<void> buf_;
  size_t len_ = 0, off_ = 0;

 public:
  deviceMemory() = default;
  static deviceMemory<T> allocate(size_t n) {
    void* p = nullptr;
    LIBP_CUDA_CHECK(cudaMalloc(&p, (n ? n : 1) * sizeof(T)));
    deviceMemory<T> m;
    m.buf_ = std::shared_ptr<void>(p, [](void* q) { cudaFree(q); });
    m.len_ = n;
    return m;
  }
  bool isInitialized() const { return buf_ != nullptr; }
  T* ptr() { return buf_ ? static_cast<T*>(buf_.get()) + off_ : nullptr; }
  const T* ptr() const { return buf_ ? static_cast<const T*>(buf_.get()) + off_ : nullptr; }
  size_t length() const { return len_; }
  size_t size() const { return len_ * sizeof(T); }
  deviceMemory<T> operator+(std::ptrdiff_t o) const {
    deviceMemory<T> m(*this);
    m.off_ += o;
    m.len_ -= o;
    return m;
  }
  void copyFrom(const memory<T> src, std::ptrdiff_t count = -1, std::ptrdiff_t offset = 0) {
    const size_t n = count < 0 ? len_ : (size_t)count;
    LIBP_ABORT("deviceMemory::copyFrom source too short", n > src.length());
    if (n) LIBP_CUDA_CHECK(cudaMemcpy(ptr() + offset, src.ptr(), n * sizeof(T),
                                      cudaMemcpyHostToDevice));
  }
  void copyTo(memory<T> dest, std::ptrdiff_t count = -1, std::ptrdiff_t offset = 0) const {
    const size_t n = count < 0 ? len_ : (size_t)count;
    LIBP_ABORT("deviceMemory::copyTo destination too short", n > dest.length());
    if (n) LIBP_CUDA_CHECK(cudaMemcpy(dest.ptr(), ptr() + offset, n * sizeof(T),
                                      cudaMemcpyDeviceToHost));
  }
  void free() {
    buf_ = nullptr;
    len_ = off_ = 0;
  }
};

// Kernel properties: the "defines/..." entries the drivers set (p_blockSize, ...).
class properties_t {
  std::map<std::string, std::string> kv_;

 public:
  // One entry, assignable from text or a number as the reference's occa::json
  // entries are (kernelInfo["defines/" "p_blockSize"] = blockSize in bs3Setup.cpp:39).
  class value {
    std::string& s_;

   public:
    explicit value(std::string& s) : s_(s) {}
    value& operator=(const std::string& v) {
      s_ = v;
      return *this;
    }
    value& operator=(const char* v) {
      s_ = v;
      return *this;
    }
    template <typename T, typename = std::enable_if_t<std::is_arithmetic<T>::value>>
    value& operator=(T v) {
      s_ = std::to_string(v);
      return *this;
    }
    operator const std::string&() const { return s_; }
  };
  value operator[](const std::string& key) { return value(kv_[key]); }
  bool has(const std::string& key) const { return kv_.count(key) != 0; }
  std::string get(const std::string& key, const std::string& dflt = "") const {
    auto it = kv_.find(key);
    return it == kv_.end() ? dflt : it->second;
  }
};

// One argument of a kernel call: an integer, a floating-point scalar or a device
// pointer (deviceMemory<T> of any T).
struct kernelArg {
  enum Kind { Int, Real, Ptr } kind;
  long long i = 0;
  double d = 0;
  void* p = nullptr;
  kernelArg(int v) : kind(Int), i(v) {}
  kernelArg(long long v) : kind(Int), i(v) {}
  kernelArg(double v) : kind(Real), d(v) {}
  kernelArg(float v) : kind(Real), d(v) {}
  template <typename T>
  kernelArg(deviceMemory<T> m) : kind(Ptr), p(static_cast<void*>(m.ptr())) {}
};

// A kernel built by platform_t::buildKernel: called with the argument list of the
// reference's OKL kernel, it runs the matching libspgb300 entry point on the
// platform's stream.
class kernel_t {
 public:
  using fn_t = sp_status (*)(const std::vector<kernelArg>&, int blockSize, cudaStream_t);
  kernel_t() = default;
  kernel_t(std::string name, fn_t fn, int blockSize, cudaStream_t stream)
      : name_(std::move(name)), fn_(fn), blockSize_(blockSize), stream_(stream) {}
  bool isInitialized() const { return fn_ != nullptr; }
  const std::string& name() const { return name_; }
  template <typename... A>
  void operator()(A... args) const {
    LIBP_ABORT("kernel not built", !fn_);
    const std::vector<kernelArg> v{kernelArg(args)...};
    checkStatus(fn_(v, blockSize_, stream_), name_.c_str());
  }

 private:
  std::string name_;
  fn_t fn_ = nullptr;
  int blockSize_ = 256;
  cudaStream_t stream_ = nullptr;
};

// The platform's device (the reference's device_t wrapper around occa::device,
// include/platform.hpp:66): this build runs OCCA's CUDA mode only.
class device_t {
  cudaStream_t* stream_ = nullptr;

 public:
  device_t() = default;
  explicit device_t(cudaStream_t* s) : stream_(s) {}
  std::string mode() const { return "CUDA"; }
  void finish() const {
    if (stream_ && *stream_) LIBP_CUDA_CHECK(cudaStreamSynchronize(*stream_));
  }
};

class platform_t {
  struct state {
    settings_t* settings = nullptr;
    properties_t props;
    cudaStream_t stream = nullptr;
    int device = 0;
  };
  std::shared_ptr<state> st_;

 public:
  comm_t comm;
  device_t device;
  platform_t() = default;
  explicit platform_t(settings_t& settings);

  bool isInitialized() const { return st_ != nullptr; }
  settings_t& settings() { return *st_->settings; }
  properties_t& props() { return st_->props; }
  cudaStream_t stream() const { return st_->stream; }
  int rank() const { return comm.rank(); }
  int size() const { return comm.size(); }

  // Binds the reference kernel `kernelName` of `fileName` (BS0-BS5 OKL files) to
  // its C-ABI entry point; p_blockSize comes from kernelInfo["defines/p_blockSize"].
  kernel_t buildKernel(const std::string& fileName, const std::string& kernelName,
                       properties_t& kernelInfo);

  template <typename T>
  deviceMemory<T> malloc(size_t count) {
    return deviceMemory<T>::allocate(count);
  }
  template <typename T>
  deviceMemory<T> malloc(size_t count, const memory<T> src) {
    deviceMemory<T> m = deviceMemory<T>::allocate(count);
    m.copyFrom(src, count);
    return m;
  }
  template <typename T>
  deviceMemory<T> malloc(const memory<T> src) {
    return malloc<T>(src.length(), src);
  }
  void finish() const { LIBP_CUDA_CHECK(cudaStreamSynchronize(st_->stream)); }
};

void platformAddSettings(settings_t& settings);
void platformReportSettings(settings_t& settings);

// include/timer.hpp: PlatformTime waits for the device; GlobalPlatformTime also
// waits for every rank (one here).
timePoint_t PlatformTime(platform_t& platform);
timePoint_t GlobalPlatformTime(platform_t& platform);

}  // namespace libp
