/*
 * Host-only stand-in for the parts of the OCCA API that the reference's headers and
 * host code name, used only to compile the reference's host code into the test
 * checker (oracle/_ref).  "Device" memory is plain host memory; kernels are never
 * launched (the checker calls the host overloads of ogs_t, which run the
 * reference's OpenMP loops).
 */
#ifndef SP_REF_SHIM_OCCA_HPP
#define SP_REF_SHIM_OCCA_HPP

#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

namespace occa {

typedef long long dim_t;
typedef unsigned long long udim_t;

class json {
 public:
  enum kind_t { none_, object_, array_, string_, number_, bool_ };
  kind_t kind = none_;
  std::string str;
  double num = 0;
  bool b = false;
  std::map<std::string, json> obj;

  json() = default;
  template <typename T>
  json(const char* key, const T& value) : kind(object_) { (*this)[key] = value; }

  json& operator[](const std::string& key) {
    kind = object_;
    const size_t slash = key.find('/');
    if (slash == std::string::npos) return obj[key];
    return obj[key.substr(0, slash)][key.substr(slash + 1)];
  }
  json& operator[](const char* key) { return (*this)[std::string(key)]; }
  json& operator=(const std::string& s) { kind = string_; str = s; return *this; }
  json& operator=(const char* s) { kind = string_; str = s; return *this; }
  json& operator=(bool v) { kind = bool_; b = v; return *this; }
  json& operator=(int v) { kind = number_; num = v; str = std::to_string(v); return *this; }
  json& operator=(long v) { kind = number_; num = (double)v; str = std::to_string(v); return *this; }
  json& operator=(long long v) { kind = number_; num = (double)v; str = std::to_string(v); return *this; }
  json& operator=(float v) { kind = number_; num = v; str = std::to_string(v); return *this; }
  json& operator=(double v) { kind = number_; num = v; str = std::to_string(v); return *this; }
  json& operator+=(const std::string& s) { kind = string_; str += s; return *this; }
  json& asObject() { if (kind == none_) kind = object_; return *this; }
  json& asArray() { if (kind == none_) kind = array_; return *this; }
  bool has(const std::string& key) const { return obj.count(key) != 0; }
  std::string toString() const { return str; }
};

class dtype_t {
 public:
  size_t bytes = 1;
  dtype_t() = default;
  explicit dtype_t(size_t b) : bytes(b) {}
};

namespace dtype {
template <typename T>
inline const dtype_t& get() {
  static const dtype_t t(sizeof(T));
  return t;
}
}  // namespace dtype

class memory {
  std::shared_ptr<char> buf;
  size_t offset_ = 0;   // bytes
  size_t size_ = 0;     // bytes
  size_t elem_ = 1;     // dtype size

 public:
  memory() = default;
  memory(std::shared_ptr<char> b, size_t bytes) : buf(std::move(b)), size_(bytes) {}

  bool isInitialized() const { return buf != nullptr; }
  void setDtype(const dtype_t& t) { elem_ = t.bytes; }
  void* ptr() { return buf ? buf.get() + offset_ : nullptr; }
  const void* ptr() const { return buf ? buf.get() + offset_ : nullptr; }
  udim_t size() const { return size_; }
  udim_t length() const { return size_ / elem_; }

  memory slice(dim_t offset, dim_t count = -1) const {
    memory m(*this);
    m.offset_ = offset_ + (size_t)offset * elem_;
    m.size_ = (count < 0) ? size_ - (size_t)offset * elem_ : (size_t)count * elem_;
    return m;
  }
  memory operator+(dim_t offset) const { return slice(offset); }

  void copyFrom(const void* src, dim_t bytes = -1, dim_t offset = 0, const json& = json()) {
    const size_t n = bytes < 0 ? size_ : (size_t)bytes;
    if (n) std::memmove((char*)ptr() + offset, src, n);
  }
  void copyFrom(const memory& src, dim_t bytes = -1, dim_t destOffset = 0, dim_t srcOffset = 0,
                const json& = json()) {
    const size_t n = bytes < 0 ? size_ : (size_t)bytes;
    if (n) std::memmove((char*)ptr() + destOffset, (const char*)src.ptr() + srcOffset, n);
  }
  void copyTo(void* dest, dim_t bytes = -1, dim_t offset = 0, const json& = json()) const {
    const size_t n = bytes < 0 ? size_ : (size_t)bytes;
    if (n) std::memmove(dest, (const char*)ptr() + offset, n);
  }
  void copyTo(memory dest, dim_t bytes = -1, dim_t destOffset = 0, dim_t srcOffset = 0,
              const json& = json()) const {
    const size_t n = bytes < 0 ? size_ : (size_t)bytes;
    if (n) std::memmove((char*)dest.ptr() + destOffset, (const char*)ptr() + srcOffset, n);
  }
  void free() {
    buf = nullptr;
    offset_ = size_ = 0;
  }
  void swap(memory& m) {
    std::swap(buf, m.buf);
    std::swap(offset_, m.offset_);
    std::swap(size_, m.size_);
    std::swap(elem_, m.elem_);
  }
};

class stream {
  bool init_ = false;

 public:
  stream() = default;
  explicit stream(bool i) : init_(i) {}
  bool isInitialized() const { return init_; }
};

class kernel {
  bool init_ = false;

 public:
  kernel() = default;
  explicit kernel(bool i) : init_(i) {}
  bool isInitialized() const { return init_; }
  template <typename... A>
  void operator()(A&&...) const {
    std::fprintf(stderr, "host-only OCCA stand-in: a device kernel was launched\n");
    std::abort();
  }
};

class device {
  std::string mode_ = "Serial";
  stream current_{true};

 public:
  device() = default;
  void setup(const json&) {}
  const std::string& mode() const { return mode_; }
  void finish() {}
  stream createStream() { return stream(true); }
  stream getStream() { return current_; }
  void setStream(const stream& s) { current_ = s; }
  template <typename T = char>
  memory malloc(size_t count, const void* src = nullptr, const json& = json()) {
    const size_t bytes = count * sizeof(T);
    std::shared_ptr<char> b(new char[bytes ? bytes : 1], std::default_delete<char[]>());
    if (src && bytes) std::memcpy(b.get(), src, bytes);
    memory m(b, bytes);
    m.setDtype(dtype::get<T>());
    return m;
  }
  template <typename T = char>
  memory malloc(size_t count, const json& props) {
    return malloc<T>(count, nullptr, props);
  }
  kernel buildKernel(const std::string&, const std::string&, const json&) { return kernel(true); }
};

inline int getDeviceCount(const std::string&) { return 0; }
namespace env {
inline void setOccaCacheDir(const std::string&) {}
}  // namespace env

}  // namespace occa

#endif
