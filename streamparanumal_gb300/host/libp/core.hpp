// libp core types for the GB300 drop-in: the names and call shapes of the
// reference's libp (include/types.h, include/utils.hpp, include/memory.hpp,
// include/comm.hpp, include/settings.hpp, include/timer.hpp) at one rank.
#pragma once

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace libp {

// include/types.h:39,52,60
#define dfloat double
#define dfloatFormat "%lf"
#define hlong long long int
#define hlongFormat "%lld"
#define dlong int
#define dlongFormat "%d"

#define LIBP_SUCCESS 0
#define LIBP_ERROR -1

// Error convention of include/utils.hpp:57-113: LIBP_ABORT(message, condition)
// throws libp::exception carrying file, function and line.
class exception : public std::runtime_error {
 public:
  exception(const std::string& file, const std::string& func, int line, const std::string& msg)
      : std::runtime_error(format(file, func, line, msg)), message(msg) {}
  std::string message;

 private:
  static std::string format(const std::string& file, const std::string& func, int line,
                            const std::string& msg) {
    std::ostringstream os;
    os << "\n---[ Error ]----------------------------------------------------------------\n"
       << "    File     : " << file << "\n    Line     : " << line << "\n    Function : " << func
       << "\n    Message  : " << msg
       << "\n============================================================================\n";
    return os.str();
  }
};

#define LIBP_ABORT(message, expr)                                                  \
  do {                                                                             \
    if (expr) {                                                                    \
      std::ostringstream _ss;                                                      \
      _ss << message;                                                              \
      throw ::libp::exception(__FILE__, __func__, __LINE__, _ss.str());            \
    }                                                                              \
  } while (0)
#define LIBP_FORCE_ABORT(message) LIBP_ABORT(message, true)

// Host array with shared ownership and offset views (include/memory.hpp:34-264).
template <typename T>
class memory {
  std::shared_ptr<T> buf_;
  size_t len_ = 0, off_ = 0;

 public:
  memory() = default;
  explicit memory(size_t n) : buf_(new T[n ? n : 1], std::default_delete<T[]>()), len_(n) {}
  memory(size_t n, const T v) : memory(n) {
    for (size_t i = 0; i < n; ++i) buf_.get()[i] = v;
  }
  void malloc(size_t n) { *this = memory<T>(n); }
  void calloc(size_t n) { *this = memory<T>(n, T{0}); }
  T* ptr() { return buf_ ? buf_.get() + off_ : nullptr; }
  const T* ptr() const { return buf_ ? buf_.get() + off_ : nullptr; }
  size_t length() const { return len_; }
  size_t size() const { return len_ * sizeof(T); }
  T& operator[](std::ptrdiff_t i) const { return buf_.get()[off_ + i]; }
  memory<T> operator+(std::ptrdiff_t o) const {
    memory<T> m(*this);
    m.off_ += o;
    m.len_ -= o;
    return m;
  }
  void free() {
    buf_ = nullptr;
    len_ = off_ = 0;
  }
};

// Single-rank communicator (include/comm.hpp): every collective is the identity.
class comm_t {
 public:
  int rank() const { return 0; }
  int size() const { return 1; }
  comm_t Dup() const { return *this; }
  void Free() {}
  void Barrier() const {}
  template <typename T>
  void Allreduce(T&) const {}
  template <typename T>
  void Allreduce(memory<T>, int = 0) const {}
};

namespace Comm {
inline void Init(int&, char**&) {}
inline void Finalize() {}
inline comm_t World() { return comm_t(); }
}  // namespace Comm

// Command-line settings registry with the reference's keys, defaults and option
// validation (include/settings.hpp:87-137, libs/core/settings.cpp:105-168).
class settings_t {
  struct setting_t {
    std::string shortkey, longkey, name, val, description;
    std::vector<std::string> options;
  };
  std::map<std::string, setting_t> settings_;
  std::vector<std::string> order_;

 public:
  comm_t comm;
  settings_t() = default;
  explicit settings_t(comm_t c) : comm(c) {}

  void newSetting(const std::string& shortkey, const std::string& longkey,
                  const std::string& name, const std::string& val,
                  const std::string& description = "",
                  const std::vector<std::string>& options = {});
  void changeSetting(const std::string& name, const std::string& val);
  void parseSettings(int argc, char** argv);
  bool hasSetting(const std::string& name) const { return settings_.count(name) != 0; }
  const std::string& raw(const std::string& name) const;
  bool compareSetting(const std::string& name, const std::string& token) const;
  void reportSetting(const std::string& name) const;
  void report() const;
  void PrintUsage() const;

  template <typename T>
  void getSetting(const std::string& name, T& value) const {
    std::istringstream is(raw(name));
    is >> value;
  }
  void getSetting(const std::string& name, std::string& value) const { value = raw(name); }
};

// Timers (include/timer.hpp:37-55): device-synchronised wall-clock time points.
using timePoint_t = std::chrono::time_point<std::chrono::steady_clock>;
timePoint_t Time();
double ElapsedTime(const timePoint_t start, const timePoint_t end);

}  // namespace libp
