// ogs_t::Setup of the GB300 drop-in: ids -> libspgb300 plan (sp_ogs_setup).
#include "ogs.hpp"

namespace libp {
namespace ogs {

namespace {
void checkKind(const Kind kind, const bool unique) {
  LIBP_ABORT("Invalid ogs setup requested",
             (kind == Unsigned && unique) || (kind == Halo && unique));
}
}  // namespace

void ogs_t::Setup(const dlong _N, memory<hlong> ids, comm_t _comm, const Kind _kind,
                  const Method, const bool _unique, const bool verbose, platform_t& _platform) {
  Free();
  platform = _platform;
  comm = _comm;
  N = _N;
  kind = _kind;
  unique = _unique;
  checkKind(kind, unique);
  const timePoint_t start = Time();
  auto holder = std::make_shared<planHolder>();
  checkStatus(sp_ogs_setup(N, reinterpret_cast<int64_t*>(ids.ptr()), (sp_kind)kind, unique ? 1 : 0,
                           (sp_stream_t)platform.stream(), &holder->p),
              "ogs_t::Setup");
  attach(holder, start, verbose);
}

void ogs_t::Setup(const dlong _N, deviceMemory<hlong> o_ids, comm_t _comm, const Kind _kind,
                  const Method, const bool _unique, const bool verbose, platform_t& _platform) {
  Free();
  platform = _platform;
  comm = _comm;
  N = _N;
  kind = _kind;
  unique = _unique;
  checkKind(kind, unique);
  const timePoint_t start = Time();
  auto holder = std::make_shared<planHolder>();
  checkStatus(sp_ogs_setup_device(N, reinterpret_cast<int64_t*>(o_ids.ptr()), (sp_kind)kind,
                                  unique ? 1 : 0, (sp_stream_t)platform.stream(), &holder->p),
              "ogs_t::Setup");
  attach(holder, start, verbose);
}

void ogs_t::attach(std::shared_ptr<planHolder> holder, const timePoint_t start,
                   const bool verbose) {
  plan_ = holder;
  sp_ogs_info info;
  checkStatus(sp_ogs_plan_info(plan(), &info), "ogs_t::Setup");
  NlocalT = info.NrowsT;
  NlocalP = info.NrowsN;
  Ngather = info.NrowsN;
  NhaloT = NhaloP = 0;
  NgatherGlobal = info.NgatherGlobal;
  if (verbose)
    std::printf("ogs Setup Time: %g seconds. (%d rows, %d warp chunks)\n",
                ElapsedTime(start, Time()), NlocalT, info.NchunksT);
}

void ogs_t::Free() {
  plan_ = nullptr;
  N = Ngather = NlocalT = NlocalP = NhaloT = NhaloP = 0;
  NgatherGlobal = 0;
}

}  // namespace ogs
}  // namespace libp
