// ogs_t::Setup of the GB300 drop-in: ids -> libspgb300 plan (sp_ogs_setup).
#include "ogs.hpp"

namespace libp {
namespace ogs {

void ogs_t::Setup(const dlong _N, memory<hlong> ids, comm_t _comm, const Kind _kind,
                  const Method, const bool _unique, const bool verbose, platform_t& _platform) {
  Free();
  platform = _platform;
  comm = _comm;
  N = _N;
  kind = _kind;
  unique = _unique;
  LIBP_ABORT("Invalid ogs setup requested",
             (kind == Unsigned && unique) || (kind == Halo && unique));
  const timePoint_t start = Time();
  auto holder = std::make_shared<planHolder>();
  checkStatus(sp_ogs_setup(N, reinterpret_cast<int64_t*>(ids.ptr()), (sp_kind)kind, unique ? 1 : 0,
                           (sp_stream_t)platform.stream(), &holder->p),
              "ogs_t::Setup");
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
