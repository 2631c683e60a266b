// Library-wide utilities: error strings, launch counter, BS0 graph objects.
#include <atomic>
#include <cstdarg>
#include <cstring>
#include <mutex>
#include <vector>

#include "sp_internal.h"

namespace sp {

static thread_local std::string t_last_error;
static thread_local int64_t t_launches = 0;

sp_status fail(sp_status s, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  t_last_error = buf;
  return s;
}

void clear_error() { t_last_error.clear(); }
void count_launch(int64_t n) { t_launches += n; }

struct TuneEntry {
  const char* name;
  int64_t lo, hi;
  std::atomic<int64_t> value;
};
// One entry per TuneKey, in the enum's order (tune(k) indexes by the key).
static TuneEntry g_tune[kTuneCount] = {
    {"reduce.prefetch_chunks", -1, 64, {-1}},
    {"ogs.block_nnz", 256, 2048, {2048}},
    {"ogs.kernel", 0, 7, {2}},
    {"ogs.order", 0, 2, {1}},
    {"reduce.rolling", 0, 1, {1}},
    {"ogs.kernel.gather", 0, 7, {2}},
    {"ogs.kernel.scatter", 0, 5, {5}},
    {"ogs.rows", 0, 1, {1}},
    {"ogs.page_shift", 3, 16, {9}},
    {"ogs.ball_shift", 0, 26, {0}},
    {"ogs.gs_order", -1, 2, {-1}},
    {"ogs.gs_page_shift", 3, 16, {8}},
    {"ogs.gs_ball_shift", 0, 26, {18}},
    {"ogs.scatter_pages", 0, 1, {1}},
    {"reduce.norm_exact", 0, 1, {0}},
    {"reduce.norm_ctas", 4, 6, {4}},
    {"reduce.norm_roll", 0, 1, {1}},
    {"ogs.singles", 0, 2, {2}},
    {"reduce.rdotr_exact", 0, 1, {0}},
    {"ogs.slabs", 0, 1, {0}},
    {"ogs.slab_seg_shift", 8, 22, {17}},
    {"ogs.slab_lane", 0, 16, {0}},
    {"ogs.slab_ctas", 0, 4, {0}},
    {"ogs.slab_load", 0, 3, {0}},
    {"ogs.slab_defer", 0, 1, {1}},
    {"ogs.slab_code_shift", 0, 12, {0}},
    {"ogs.kernel.f32", -1, 7, {-1}},
    {"ogs.kernel.gather.f32", -1, 7, {-1}},
    {"ogs.slab_row_codes", 0, 1, {0}},
};

int64_t tune(TuneKey k) { return g_tune[k].value.load(std::memory_order_relaxed); }

int sm_count() {
  static std::mutex mu;
  static std::vector<int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 152;
  std::lock_guard<std::mutex> lock(mu);
  if ((int)cache.size() <= dev) cache.resize(dev + 1, 0);
  if (cache[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 152;
    cache[dev] = n;
  }
  return cache[dev];
}

}  // namespace sp

extern "C" {

const char* sp_last_error_string(void) { return sp::t_last_error.c_str(); }

const char* sp_status_string(sp_status s) {
  switch (s) {
    case SP_SUCCESS: return "success";
    case SP_ERR_INVALID_ARG: return "invalid argument";
    case SP_ERR_CUDA: return "CUDA error";
    case SP_ERR_ALLOC: return "allocation failed";
    case SP_ERR_UNSUPPORTED: return "unsupported combination";
    case SP_ERR_SIZE: return "size limit exceeded";
    case SP_ERR_CSR: return "malformed CSR or ids";
    case SP_ERR_TIMEOUT: return "device wait timed out";
    case SP_ERR_DEVICE_CHECK: return "device bounds check failed";
    default: return "unknown status";
  }
}

int32_t sp_version(void) { return 100; }  // 0.1.0

int64_t sp_launch_count(void) { return sp::t_launches; }

sp_status sp_tune_set(const char* key, int64_t value) {
  if (!key) return sp::fail(SP_ERR_INVALID_ARG, "sp_tune_set: null key");
  for (auto& e : sp::g_tune)
    if (std::strcmp(e.name, key) == 0) {
      if (value < e.lo || value > e.hi)
        return sp::fail(SP_ERR_INVALID_ARG, "sp_tune_set: %s=%lld outside [%lld, %lld]", key,
                        (long long)value, (long long)e.lo, (long long)e.hi);
      e.value.store(value, std::memory_order_relaxed);
      return SP_SUCCESS;
    }
  return sp::fail(SP_ERR_INVALID_ARG, "sp_tune_set: unknown key '%s'", key);
}

sp_status sp_tune_get(const char* key, int64_t* value) {
  if (!key || !value) return sp::fail(SP_ERR_INVALID_ARG, "sp_tune_get: null argument");
  for (auto& e : sp::g_tune)
    if (std::strcmp(e.name, key) == 0) {
      *value = e.value.load(std::memory_order_relaxed);
      return SP_SUCCESS;
    }
  return sp::fail(SP_ERR_INVALID_ARG, "sp_tune_get: unknown key '%s'", key);
}
void sp_launch_count_reset(void) { sp::t_launches = 0; }

}  // extern "C"
