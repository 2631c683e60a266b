// Multi-rank gather-scatter handle: the local and halo operators of one rank and
// the pairwise exchange schedules that join the halo rows across ranks.
#pragma once

#include <cstdint>
#include <vector>

#include "sp_internal.h"

// One transpose mode of the pairwise exchange (the reference's ogsPairwise_t::data_t,
// include/ogs/ogsExchange.hpp:166-239).
struct SpMrSched {
  int32_t Nsend = 0;   // gathered halo rows packed into the send buffer
  int32_t NrowsP = 0;  // own rows at the head of the halo buffer
  int32_t Nrows = 0;   // rows of the post-exchange gather
  int32_t Ncols = 0;   // NrowsP + entries received
  std::vector<int32_t> sendRanks, sendCounts, sendOffsets;
  std::vector<int32_t> recvRanks, recvCounts, recvOffsets;
  std::vector<int32_t> sendIds;         // Nsend halo rows, grouped by destination
  std::vector<int32_t> postRs, postCi;  // CSR: Nrows + 1, Ncols
  int32_t* d_sendIds = nullptr;
  sp_ogs_plan* post = nullptr;
};

struct sp_ogs_mr {
  int32_t N = 0;
  int32_t kind = SP_KIND_SIGNED;
  int32_t NlocalP = 0, NlocalT = 0, NhaloP = 0, NhaloT = 0, Nshared = 0;
  int64_t NgatherGlobal = 0;
  int32_t gather_defined = 1;
  // host CSR of the local and halo operators: T (all members) and N (positive)
  std::vector<int32_t> csr[2][4];  // [local|halo][rsT, ciT, rsN, ciN]
  sp_ogs_plan* op[2] = {nullptr, nullptr};
  SpMrSched sched[3];  // indexed by sp_transpose: Sym, NoTrans, Trans
  int device = -1;
};

namespace sp {
// Device half of the setup: operators, post-exchange gathers and send lists.
sp_status mr_upload(sp_ogs_mr* h, cudaStream_t s);
// Releases every device resource of the handle.
void mr_free_device(sp_ogs_mr* h);
}  // namespace sp
