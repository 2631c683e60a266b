// ogs::ogs_t of the GB300 drop-in at one rank: the reference's API
// (include/ogs.hpp:177-344) over a libspgb300 gather-scatter plan.  Device-buffer
// overloads launch the CUDA kernels on the platform's stream; host-buffer overloads
// stage through the device and run the same kernels (there is no CPU path).
#pragma once

#include <type_traits>

#include "platform.hpp"

namespace libp {
namespace ogs {

typedef enum { Float, Double, Int32, Int64 } Type;
typedef enum { Add, Mul, Max, Min } Op;
typedef enum { Sym, NoTrans, Trans } Transpose;
typedef enum { Auto, Pairwise, CrystalRouter, AllToAll } Method;
typedef enum { Unsigned, Signed, Halo } Kind;

template <typename T>
constexpr Type ogsType() {
  return std::is_same<T, float>::value      ? Float
         : std::is_same<T, double>::value   ? Double
         : std::is_same<T, int>::value      ? Int32
                                            : Int64;
}

class ogs_t {
 public:
  platform_t platform;
  comm_t comm;
  dlong N = 0, Ngather = 0, NlocalT = 0, NlocalP = 0, NhaloT = 0, NhaloP = 0;
  hlong NgatherGlobal = 0;
  Kind kind = Signed;
  bool unique = false;

  ogs_t() = default;

  void Setup(const dlong _N, memory<hlong> ids, comm_t _comm, const Kind _kind,
             const Method method, const bool _unique, const bool verbose,
             platform_t& _platform);
  // The same setup from ids already in device memory (grouped on the GPU by
  // sp_ogs_setup_device; unique signs written back into o_ids).
  void Setup(const dlong _N, deviceMemory<hlong> o_ids, comm_t _comm, const Kind _kind,
             const Method method, const bool _unique, const bool verbose,
             platform_t& _platform);
  void Free();
  sp_ogs_plan* plan() const { return plan_ ? plan_->p : nullptr; }

  template <typename T>
  void GatherScatter(deviceMemory<T> o_v, const int k, const Op op, const Transpose trans) {
    GatherScatterStart(o_v, k, op, trans);
    GatherScatterFinish(o_v, k, op, trans);
  }
  template <typename T>
  void GatherScatterStart(deviceMemory<T>, const int, const Op, const Transpose) {
    need();  // one rank: no halo to pack
  }
  template <typename T>
  void GatherScatterFinish(deviceMemory<T> o_v, const int k, const Op op,
                           const Transpose trans) {
    need();
    checkStatus(sp_ogs_gather_scatter(plan(), (sp_type)ogsType<T>(), (sp_op)op,
                                      (sp_transpose)trans, k, o_v.ptr(),
                                      (sp_stream_t)platform.stream()),
                "ogs_t::GatherScatter");
  }

  template <typename T>
  void Gather(deviceMemory<T> o_gv, deviceMemory<T> o_v, const int k, const Op op,
              const Transpose trans) {
    GatherStart(o_gv, o_v, k, op, trans);
    GatherFinish(o_gv, o_v, k, op, trans);
  }
  template <typename T>
  void GatherStart(deviceMemory<T>, deviceMemory<T>, const int, const Op, const Transpose) {
    need();
  }
  template <typename T>
  void GatherFinish(deviceMemory<T> o_gv, deviceMemory<T> o_v, const int k, const Op op,
                    const Transpose trans) {
    need();
    checkStatus(sp_ogs_gather(plan(), (sp_type)ogsType<T>(), (sp_op)op, (sp_transpose)trans, k,
                              o_gv.ptr(), o_v.ptr(), (sp_stream_t)platform.stream()),
                "ogs_t::Gather");
  }

  template <typename T>
  void Scatter(deviceMemory<T> o_v, deviceMemory<T> o_gv, const int k, const Transpose trans) {
    ScatterStart(o_v, o_gv, k, trans);
    ScatterFinish(o_v, o_gv, k, trans);
  }
  template <typename T>
  void ScatterStart(deviceMemory<T>, deviceMemory<T>, const int, const Transpose) {
    need();
  }
  template <typename T>
  void ScatterFinish(deviceMemory<T> o_v, deviceMemory<T> o_gv, const int k,
                     const Transpose trans) {
    need();
    checkStatus(sp_ogs_scatter(plan(), (sp_type)ogsType<T>(), (sp_transpose)trans, k, o_v.ptr(),
                               o_gv.ptr(), (sp_stream_t)platform.stream()),
                "ogs_t::Scatter");
  }

  // host-buffer overloads: staged through the device
  template <typename T>
  void GatherScatter(memory<T> v, const int k, const Op op, const Transpose trans) {
    deviceMemory<T> o_v = platform.malloc<T>((size_t)N * k, v);
    GatherScatter(o_v, k, op, trans);
    o_v.copyTo(v, (size_t)N * k);
  }
  template <typename T>
  void Gather(memory<T> gv, const memory<T> v, const int k, const Op op, const Transpose trans) {
    const size_t rows = (trans == NoTrans) ? NlocalP : NlocalT;
    deviceMemory<T> o_v = platform.malloc<T>((size_t)N * k, v);
    deviceMemory<T> o_gv = platform.malloc<T>(rows * k);
    Gather(o_gv, o_v, k, op, trans);
    o_gv.copyTo(gv, rows * k);
  }
  template <typename T>
  void Scatter(memory<T> v, const memory<T> gv, const int k, const Transpose trans) {
    const size_t rows = (trans == Trans) ? NlocalP : NlocalT;
    deviceMemory<T> o_v = platform.malloc<T>((size_t)N * k, v);
    deviceMemory<T> o_gv = platform.malloc<T>(rows * k, gv);
    Scatter(o_v, o_gv, k, trans);
    o_v.copyTo(v, (size_t)N * k);
  }

 private:
  struct planHolder {
    sp_ogs_plan* p = nullptr;
    ~planHolder() { sp_ogs_plan_destroy(p); }
  };
  std::shared_ptr<planHolder> plan_;
  void need() const { LIBP_ABORT("ogs handle is not set up.", !plan_); }
  void attach(std::shared_ptr<planHolder> holder, const timePoint_t start, const bool verbose);
};

}  // namespace ogs
}  // namespace libp
