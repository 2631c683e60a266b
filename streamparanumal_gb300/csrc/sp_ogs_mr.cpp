// Multi-rank gather-scatter setup on the host: which groups are shared between
// ranks, the local / halo split, the shared-node lists and the pairwise exchange
// schedules.  All communication goes through the caller's sp_comm callbacks.
//
// Steps (ogsBase_t::Setup, libs/ogs/ogsSetup.cpp:87-290):
//  1. every non-zero id is sent to its home rank |id| % size, which groups the
//     copies by |id|: a group is shared when its copies come from more than one rank.
//     With `unique` the home rank makes one copy positive, drawing from the LCG
//     seeded with its rank (FindSharedGroups, :292-469);
//  2. the ids split into a local and a halo id set, each turned into an operator
//     with the one-rank rules (rows by first appearance, positive rows first);
//  3. each halo row is sent to the home rank of its id, which returns to every
//     participant the (rank, row, sign) of all other participants
//     (ConstructSharedNodes, :617-813);
//  4. for each transpose mode the shared pairs are sorted by peer rank into a send
//     list, the peers learn which of their rows each value lands in, and the
//     post-exchange gather puts each row's own value first and the received values
//     after it in ascending rank order (ogsPairwise_t, ogsPairwise.cpp:176-387).
// Every rank runs the same sequence of collectives, also after a local error: an
// error flag is reduced at the end, so that all ranks fail together.
#include <parallel/algorithm>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <vector>

#include "sp_ogs_mr.h"
#include "sp_ogs_plan.h"

namespace sp {
namespace {

struct CommFailure : std::runtime_error {
  using std::runtime_error::runtime_error;
};

inline int64_t iabs(int64_t v) { return v < 0 ? -v : v; }

std::vector<int64_t> prefix(const std::vector<int64_t>& c) {
  std::vector<int64_t> o(c.size() + 1, 0);
  for (size_t i = 0; i < c.size(); ++i) o[i + 1] = o[i] + c[i];
  return o;
}

class Comm {
 public:
  explicit Comm(const sp_comm& c) : c_(c) {}
  int rank() const { return c_.rank; }
  int size() const { return c_.size; }

  // counts[r] to rank r -> the counts every rank addressed to this one
  std::vector<int64_t> counts(const std::vector<int64_t>& send) {
    const int P = size();
    std::vector<int64_t> one(P, 1), disp(P), recv(P, 0);
    std::iota(disp.begin(), disp.end(), 0);
    raw(send.data(), one.data(), disp.data(), recv.data(), one.data(), disp.data(), 8);
    return recv;
  }

  template <class T>
  std::vector<T> alltoallv(const std::vector<T>& send, const std::vector<int64_t>& scount,
                           const std::vector<int64_t>& rcount) {
    const std::vector<int64_t> sd = prefix(scount), rd = prefix(rcount);
    std::vector<T> recv((size_t)rd.back());
    // non-null buffers even when nothing moves
    T dummy_s{}, dummy_r{};
    raw(send.empty() ? &dummy_s : send.data(), scount.data(), sd.data(),
        recv.empty() ? &dummy_r : recv.data(), rcount.data(), rd.data(), (int32_t)sizeof(T));
    return recv;
  }

  int64_t allreduce(int64_t v, int op) {
    if (c_.allreduce_i64(c_.ctx, &v, op) != 0) throw CommFailure("allreduce_i64 failed");
    return v;
  }

 private:
  void raw(const void* s, const int64_t* sc, const int64_t* sd, void* r, const int64_t* rc,
           const int64_t* rd, int32_t eb) {
    if (c_.alltoallv(c_.ctx, s, sc, sd, r, rc, rd, eb) != 0) throw CommFailure("alltoallv failed");
  }
  sp_comm c_;
};

constexpr int kLocal = 1, kShared = 2;

// Stable order of positions [0, n) by key(i).
template <class Key>
std::vector<int64_t> stable_order(int64_t n, Key key) {
  std::vector<int64_t> o((size_t)n);
  std::iota(o.begin(), o.end(), 0);
  __gnu_parallel::stable_sort(o.begin(), o.end(),
                              [&](int64_t a, int64_t b) { return key(a) < key(b); });
  return o;
}

// Rank of each received entry (entries arrive grouped by source rank).
std::vector<int32_t> sources(const std::vector<int64_t>& rcount) {
  std::vector<int32_t> src;
  for (size_t r = 0; r < rcount.size(); ++r) src.insert(src.end(), (size_t)rcount[r], (int32_t)r);
  return src;
}

// Builds one operator from the ids of one part (others zeroed) with the one-rank rules.
sp_status part_csr(int32_t N, const std::vector<int64_t>& sub, sp_kind kind,
                   std::vector<int32_t>* csr, int32_t* NrowsT, int32_t* NrowsN) {
  csr[0].assign((size_t)N + 1, 0);
  csr[1].assign((size_t)std::max(N, 1), 0);
  csr[2].assign((size_t)N + 1, 0);
  csr[3].assign((size_t)std::max(N, 1), 0);
  sp_status st = sp_ogs_setup_csr(N, const_cast<int64_t*>(sub.data()), kind, 0, NrowsT,
                                  csr[0].data(), csr[1].data(), NrowsN, csr[2].data(),
                                  csr[3].data());
  if (st) return st;
  csr[0].resize((size_t)*NrowsT + 1);
  csr[1].resize((size_t)csr[0].back());
  csr[2].resize((size_t)*NrowsN + 1);
  csr[3].resize((size_t)csr[2].back());
  return SP_SUCCESS;
}

struct SharedPair {
  int32_t rank;       // remote rank
  int32_t localRow;   // halo row here
  int32_t remoteRow;  // halo row there
  int64_t remoteId;   // signed id there
};

// Pairwise schedule of one mode from the pairs (already sorted by rank, then row).
void build_schedule(Comm& comm, const std::vector<SharedPair>& pairs,
                    const std::vector<uint8_t>& take, int32_t NrowsP, int32_t Nrows,
                    SpMrSched& x, int& bad) {
  const int P = comm.size();
  std::vector<int64_t> scount(P, 0);
  std::vector<int32_t> remoteRows;
  x.sendIds.clear();
  for (size_t i = 0; i < pairs.size(); ++i)
    if (take[i]) {
      ++scount[pairs[i].rank];
      x.sendIds.push_back(pairs[i].localRow);
      remoteRows.push_back(pairs[i].remoteRow);
    }
  const std::vector<int64_t> rcount = comm.counts(scount);
  const std::vector<int32_t> recvRows = comm.alltoallv(remoteRows, scount, rcount);
  x.Nsend = (int32_t)x.sendIds.size();
  x.NrowsP = NrowsP;
  x.Nrows = Nrows;
  x.Ncols = NrowsP + (int32_t)recvRows.size();
  // columns: own rows 0..NrowsP-1, then the received values; stable by row
  std::vector<int32_t> rowOf((size_t)x.Ncols);
  for (int32_t c = 0; c < NrowsP; ++c) rowOf[c] = c;
  for (size_t j = 0; j < recvRows.size(); ++j) {
    int32_t r = recvRows[j];
    if (r < 0 || r >= Nrows) {
      bad = 1;
      r = 0;
    }
    rowOf[NrowsP + j] = r;
  }
  x.postRs.assign((size_t)Nrows + 1, 0);
  for (int32_t c = 0; c < x.Ncols; ++c) ++x.postRs[(size_t)rowOf[c] + 1];
  if (Nrows == 0 && x.Ncols > 0) bad = 1;
  for (int32_t r = 0; r < Nrows; ++r) x.postRs[r + 1] += x.postRs[r];
  x.postCi.assign((size_t)x.Ncols, 0);
  if (Nrows > 0) {
    std::vector<int32_t> fill(x.postRs.begin(), x.postRs.end() - 1);
    for (int32_t c = 0; c < x.Ncols; ++c) x.postCi[fill[rowOf[c]]++] = c;
  }
  const std::vector<int64_t> so = prefix(scount), ro = prefix(rcount);
  x.sendRanks.clear(); x.sendCounts.clear(); x.sendOffsets.clear();
  x.recvRanks.clear(); x.recvCounts.clear(); x.recvOffsets.clear();
  for (int r = 0; r < P; ++r) {
    if (scount[r] > 0) {
      x.sendRanks.push_back(r);
      x.sendCounts.push_back((int32_t)scount[r]);
      x.sendOffsets.push_back((int32_t)so[r]);
    }
    if (rcount[r] > 0) {
      x.recvRanks.push_back(r);
      x.recvCounts.push_back((int32_t)rcount[r]);
      x.recvOffsets.push_back((int32_t)ro[r]);
    }
  }
}

sp_status mr_setup_host(int32_t N, int64_t* ids, sp_kind kind, int32_t unique, Comm& comm,
                        sp_ogs_mr* h) {
  const int P = comm.size(), me = comm.rank();
  h->N = N;
  h->kind = kind;
  int bad = 0;  // a local inconsistency; reduced over the ranks at the end

  // ---- 1. shared groups (and owners) at the home ranks
  std::vector<int32_t> nz;
  for (int32_t l = 0; l < N; ++l)
    if (ids[l] != 0) nz.push_back(l);
  const int64_t Nids = (int64_t)nz.size();
  std::vector<int64_t> scount(P, 0);
  for (int32_t l : nz) ++scount[iabs(ids[l]) % P];
  std::vector<int64_t> sendPos(P);
  {
    const std::vector<int64_t> so = prefix(scount);
    std::copy(so.begin(), so.end() - 1, sendPos.begin());
  }
  std::vector<int64_t> sendIdx((size_t)Nids), sendIds((size_t)Nids);
  for (int64_t i = 0; i < Nids; ++i) {
    const int64_t pos = sendPos[iabs(ids[nz[i]]) % P]++;
    sendIdx[pos] = i;
    sendIds[pos] = ids[nz[i]];
  }
  const std::vector<int64_t> rcount = comm.counts(scount);
  std::vector<int64_t> recvIds = comm.alltoallv(sendIds, scount, rcount);
  const std::vector<int32_t> src = sources(rcount);
  const int64_t recvN = (int64_t)recvIds.size();
  const std::vector<int64_t> byId = stable_order(recvN, [&](int64_t j) { return iabs(recvIds[j]); });
  std::vector<int32_t> recvFlag((size_t)recvN, kLocal);
  int64_t wellDefined = 1;
  Lcg rng((uint64_t)me);  // seedRNG(rank), ogsSetup.cpp:109
  for (int64_t a = 0; a < recvN;) {
    const int64_t key = iabs(recvIds[byId[a]]);
    int64_t b = a + 1;
    while (b < recvN && iabs(recvIds[byId[b]]) == key) ++b;
    int flag = kLocal;
    for (int64_t i = a + 1; i < b; ++i)
      if (src[byId[i]] != src[byId[a]]) flag = kShared;
    for (int64_t i = a; i < b; ++i) recvFlag[byId[i]] = flag;
    if (unique) {
      const int32_t m = rng.next_int() % (int32_t)(b - a);
      for (int64_t i = a; i < b; ++i) recvIds[byId[i]] = -key;
      if (m >= 0) recvIds[byId[a + m]] = key;
    } else {
      int positives = 0;
      for (int64_t i = a; i < b; ++i) positives += recvIds[byId[i]] > 0;
      if (positives != 1) wellDefined = 0;
    }
    a = b;
  }
  const std::vector<int32_t> backFlag = comm.alltoallv(recvFlag, rcount, scount);
  std::vector<int32_t> flag((size_t)Nids, kLocal);
  for (int64_t pos = 0; pos < Nids; ++pos) flag[sendIdx[pos]] = backFlag[pos];
  if (unique) {
    const std::vector<int64_t> backIds = comm.alltoallv(recvIds, rcount, scount);
    for (int64_t pos = 0; pos < Nids; ++pos) ids[nz[sendIdx[pos]]] = backIds[pos];
  }
  h->gather_defined = (int32_t)comm.allreduce(wellDefined, 1);

  // ---- 2. local and halo operators
  const sp_kind knd = (kind == SP_KIND_UNSIGNED) ? SP_KIND_UNSIGNED : SP_KIND_SIGNED;
  std::vector<int64_t> sub((size_t)N, 0);
  int32_t rowsT[2] = {0, 0}, rowsN[2] = {0, 0};
  for (int part = 0; part < 2; ++part) {
    std::fill(sub.begin(), sub.end(), 0);
    for (int64_t i = 0; i < Nids; ++i)
      if (flag[i] == (part == 0 ? kLocal : kShared)) sub[nz[i]] = ids[nz[i]];
    if (part_csr(N, sub, knd, h->csr[part], &rowsT[part], &rowsN[part])) bad = 1;
  }
  h->NlocalT = rowsT[0];
  h->NlocalP = rowsN[0];
  h->NhaloT = rowsT[1];
  h->NhaloP = rowsN[1];

  // ---- 3. shared nodes: every participant of a halo group learns the others
  const std::vector<int32_t>& hrs = h->csr[1][0];
  const std::vector<int32_t>& hci = h->csr[1][1];
  const int32_t NhaloT = h->NhaloT, NhaloP = h->NhaloP;
  std::vector<int64_t> rowId((size_t)NhaloT);
  for (int32_t n = 0; n < NhaloT; ++n) {
    const int64_t key = iabs(ids[hci[hrs[n]]]);
    rowId[n] = (n < NhaloP) ? key : -key;
  }
  std::vector<int64_t> sc2(P, 0);
  for (int32_t n = 0; n < NhaloT; ++n) ++sc2[iabs(rowId[n]) % P];
  std::vector<int64_t> pos2(P);
  {
    const std::vector<int64_t> so = prefix(sc2);
    std::copy(so.begin(), so.end() - 1, pos2.begin());
  }
  std::vector<int64_t> sId2((size_t)NhaloT);
  std::vector<int32_t> sRow2((size_t)NhaloT);
  for (int32_t n = 0; n < NhaloT; ++n) {
    const int64_t pos = pos2[iabs(rowId[n]) % P]++;
    sId2[pos] = rowId[n];
    sRow2[pos] = n;
  }
  const std::vector<int64_t> rc2 = comm.counts(sc2);
  const std::vector<int64_t> rId2 = comm.alltoallv(sId2, sc2, rc2);
  const std::vector<int32_t> rRow2 = comm.alltoallv(sRow2, sc2, rc2);
  const std::vector<int32_t> src2 = sources(rc2);
  const int64_t recvN2 = (int64_t)rId2.size();
  const std::vector<int64_t> byId2 = stable_order(recvN2, [&](int64_t j) { return iabs(rId2[j]); });
  std::vector<int64_t> grpA((size_t)recvN2), grpB((size_t)recvN2);  // group range in byId2
  for (int64_t a = 0; a < recvN2;) {
    const int64_t key = iabs(rId2[byId2[a]]);
    int64_t b = a + 1;
    while (b < recvN2 && iabs(rId2[byId2[b]]) == key) ++b;
    for (int64_t i = a; i < b; ++i) {
      grpA[byId2[i]] = a;
      grpB[byId2[i]] = b;
    }
    a = b;
  }
  // replies, in receive order (so grouped by the rank they go back to)
  std::vector<int64_t> repCount(P, 0);
  std::vector<int32_t> repRank, repLocalRow, repRemoteRow;
  std::vector<int64_t> repRemoteId;
  for (int64_t j = 0; j < recvN2; ++j)
    for (int64_t i = grpA[j]; i < grpB[j]; ++i) {
      const int64_t o = byId2[i];
      if (o == j) continue;
      ++repCount[src2[j]];
      repRank.push_back(src2[o]);
      repRemoteId.push_back(rId2[o]);
      repRemoteRow.push_back(rRow2[o]);
      repLocalRow.push_back(rRow2[j]);
    }
  const std::vector<int64_t> rc3 = comm.counts(repCount);
  const std::vector<int32_t> shRank = comm.alltoallv(repRank, repCount, rc3);
  const std::vector<int64_t> shRemoteId = comm.alltoallv(repRemoteId, repCount, rc3);
  const std::vector<int32_t> shLocalRow = comm.alltoallv(repLocalRow, repCount, rc3);
  const std::vector<int32_t> shRemoteRow = comm.alltoallv(repRemoteRow, repCount, rc3);
  const int64_t Nshared = (int64_t)shRank.size();
  h->Nshared = (int32_t)Nshared;

  // ---- 4. pairwise schedules: pairs by peer rank, then by local row (each
  // (peer, row) pair is unique: a rank has one halo row per shared group)
  std::vector<SharedPair> pairs((size_t)Nshared);
  for (int64_t i = 0; i < Nshared; ++i) {
    pairs[i] = {shRank[i], shLocalRow[i], shRemoteRow[i], shRemoteId[i]};
    if (shLocalRow[i] < 0 || shLocalRow[i] >= NhaloT || shRank[i] < 0 || shRank[i] >= P) bad = 1;
  }
  std::stable_sort(pairs.begin(), pairs.end(), [](const SharedPair& a, const SharedPair& b) {
    return a.rank != b.rank ? a.rank < b.rank : a.localRow < b.localRow;
  });
  std::vector<uint8_t> take((size_t)Nshared, 1);
  build_schedule(comm, pairs, take, NhaloT, NhaloT, h->sched[SP_SYM], bad);
  if (knd == SP_KIND_SIGNED) {
    // NoTrans: values of rows positive here go to every other participant
    for (int64_t i = 0; i < Nshared; ++i) take[i] = pairs[i].localRow < NhaloP;
    build_schedule(comm, pairs, take, NhaloP, NhaloT, h->sched[SP_NOTRANS], bad);
    // Trans: every participant sends its partial to the positive owner
    for (int64_t i = 0; i < Nshared; ++i) take[i] = pairs[i].remoteId > 0;
    build_schedule(comm, pairs, take, NhaloP, NhaloP, h->sched[SP_TRANS], bad);
  } else {
    h->sched[SP_NOTRANS] = h->sched[SP_SYM];
    h->sched[SP_TRANS] = h->sched[SP_SYM];
  }

  h->NgatherGlobal = comm.allreduce((int64_t)h->NlocalP + h->NhaloP, 0);
  if (comm.allreduce(bad, 2) != 0)
    return fail(SP_ERR_CSR, "sp_ogs_mr_setup: inconsistent ids or exchange lists across ranks");
  if (kind == SP_KIND_HALO && !h->gather_defined)
    return fail(SP_ERR_INVALID_ARG,
                "Halo exchange not well-defined. Some baseId groups have no unique positive id.");
  return SP_SUCCESS;
}

// ---- rank grid of the box mesh (Factor3 / RankDecomp3, libs/core/rankDecomp.cpp)
int largest_prime_factor(int n) {
  int best = 1;
  for (int f = 2; (int64_t)f * f <= n; ++f)
    while (n % f == 0) {
      best = f;
      n /= f;
    }
  return n > 1 ? n : best;
}

// size = sx*sy*sz with sx >= sy >= sz close to one another: the first divisor
// from round(cbrt(size)) upwards, its cofactor split the same way from round(sqrt).
void factor3(int n, int& sx, int& sy, int& sz) {
  sy = sz = 1;
  for (sx = (int)std::lround(std::cbrt((double)n)); sx < n; ++sx) {
    if (n % sx) continue;
    const int f = n / sx;
    for (sy = (int)std::lround(std::sqrt((double)f)); sy < f; ++sy)
      if (f % sy == 0) {
        sz = f / sy;
        int v[3] = {sx, sy, sz};
        std::sort(v, v + 3, [](int a, int b) { return a > b; });
        sx = v[0]; sy = v[1]; sz = v[2];
        return;
      }
    sy = f;
    sz = 1;
    if (sy > sx) std::swap(sx, sy);
    return;
  }
  sx = n;
}

// Rank coordinates: split the largest dimension by its largest prime factor p; the
// rank's slab is rank / (size/p) and the rest recurses on rank % (size/p).
void rank_coords(int sx, int sy, int sz, int rank, int& rx, int& ry, int& rz) {
  const int size = sx * sy * sz;
  if (size == 1) {
    rx = ry = rz = 0;
    return;
  }
  if (sz >= sx && sz >= sy) {
    const int p = largest_prime_factor(sz), cs = size / p;
    rank_coords(sx, sy, sz / p, rank % cs, rx, ry, rz);
    rz += (rank / cs) * (sz / p);
  } else if (sy >= sx && sy >= sz) {
    const int p = largest_prime_factor(sy), cs = size / p;
    rank_coords(sx, sy / p, sz, rank % cs, rx, ry, rz);
    ry += (rank / cs) * (sy / p);
  } else {
    const int p = largest_prime_factor(sx), cs = size / p;
    rank_coords(sx / p, sy, sz, rank % cs, rx, ry, rz);
    rx += (rank / cs) * (sx / p);
  }
}

}  // namespace
}  // namespace sp

using namespace sp;

extern "C" {

sp_status sp_ogs_mr_setup(int32_t N, int64_t* ids, sp_kind kind, int32_t unique,
                          const sp_comm* comm, int32_t upload, sp_stream_t stream,
                          sp_ogs_mr** out) {
  if (!out) return fail(SP_ERR_INVALID_ARG, "sp_ogs_mr_setup: null out");
  *out = nullptr;
  if (!comm || !comm->alltoallv || !comm->allreduce_i64 || comm->size < 1 || comm->rank < 0 ||
      comm->rank >= comm->size)
    return fail(SP_ERR_INVALID_ARG, "sp_ogs_mr_setup: bad communicator");
  if (N < 0 || (N > 0 && !ids)) return fail(SP_ERR_INVALID_ARG, "sp_ogs_mr_setup: bad ids");
  if (kind < SP_KIND_UNSIGNED || kind > SP_KIND_HALO)
    return fail(SP_ERR_INVALID_ARG, "sp_ogs_mr_setup: bad kind");
  if ((kind == SP_KIND_UNSIGNED && unique) || (kind == SP_KIND_HALO && unique))
    return fail(SP_ERR_INVALID_ARG, "Invalid ogs setup requested");
  sp_ogs_mr* h = new sp_ogs_mr();
  sp_status st;
  try {
    Comm c(*comm);
    st = mr_setup_host(N, ids, kind, unique, c, h);
  } catch (const CommFailure& e) {
    st = fail(SP_ERR_COMM, "sp_ogs_mr_setup: %s", e.what());
  } catch (const std::bad_alloc&) {
    st = fail(SP_ERR_ALLOC, "sp_ogs_mr_setup: host allocation failed");
  }
  if (!st && upload) st = mr_upload(h, as_cuda(stream));
  if (st) {
    mr_free_device(h);
    delete h;
    return st;
  }
  *out = h;
  return SP_SUCCESS;
}

sp_status sp_ogs_mr_destroy(sp_ogs_mr* h) {
  if (!h) return SP_SUCCESS;
  mr_free_device(h);
  delete h;
  return SP_SUCCESS;
}

sp_status sp_ogs_mr_info_get(const sp_ogs_mr* h, sp_ogs_mr_info* info) {
  if (!h || !info) return fail(SP_ERR_INVALID_ARG, "sp_ogs_mr_info_get: null argument");
  info->N = h->N;
  info->NlocalP = h->NlocalP;
  info->NlocalT = h->NlocalT;
  info->NhaloP = h->NhaloP;
  info->NhaloT = h->NhaloT;
  info->Nshared = h->Nshared;
  info->gather_defined = h->gather_defined;
  info->uploaded = h->op[0] != nullptr;
  info->Ngather = (int64_t)h->NlocalP + h->NhaloP;
  info->NgatherGlobal = h->NgatherGlobal;
  return SP_SUCCESS;
}

const sp_ogs_plan* sp_ogs_mr_plan(const sp_ogs_mr* h, int32_t which) {
  if (!h || which < 0 || which > 1) return nullptr;
  return h->op[which];
}

sp_status sp_ogs_mr_csr(const sp_ogs_mr* h, int32_t which, sp_transpose op, int32_t* rowStarts,
                        int32_t* colIds) {
  if (!h || which < 0 || which > 1 || (op != SP_TRANS && op != SP_NOTRANS))
    return fail(SP_ERR_INVALID_ARG, "sp_ogs_mr_csr: bad arguments");
  const int t = (op == SP_TRANS) ? 0 : 2;
  const std::vector<int32_t>& rs = h->csr[which][t];
  const std::vector<int32_t>& ci = h->csr[which][t + 1];
  if (rowStarts) std::copy(rs.begin(), rs.end(), rowStarts);
  if (colIds) std::copy(ci.begin(), ci.end(), colIds);
  return SP_SUCCESS;
}

sp_status sp_ogs_mr_schedule(const sp_ogs_mr* h, sp_transpose mode, sp_ogs_mr_sched* s,
                             int32_t* sendRanks, int32_t* sendCounts, int32_t* sendOffsets,
                             int32_t* recvRanks, int32_t* recvCounts, int32_t* recvOffsets,
                             int32_t* sendIds, int32_t* postRowStarts, int32_t* postColIds) {
  if (!h || !s || mode < SP_SYM || mode > SP_TRANS)
    return fail(SP_ERR_INVALID_ARG, "sp_ogs_mr_schedule: bad arguments");
  const SpMrSched& x = h->sched[mode];
  s->Nsend = x.Nsend;
  s->NrowsP = x.NrowsP;
  s->Nrows = x.Nrows;
  s->Ncols = x.Ncols;
  s->NranksSend = (int32_t)x.sendRanks.size();
  s->NranksRecv = (int32_t)x.recvRanks.size();
  auto put = [](const std::vector<int32_t>& v, int32_t* d) {
    if (d) std::copy(v.begin(), v.end(), d);
  };
  put(x.sendRanks, sendRanks);
  put(x.sendCounts, sendCounts);
  put(x.sendOffsets, sendOffsets);
  put(x.recvRanks, recvRanks);
  put(x.recvCounts, recvCounts);
  put(x.recvOffsets, recvOffsets);
  put(x.sendIds, sendIds);
  put(x.postRs, postRowStarts);
  put(x.postCi, postColIds);
  return SP_SUCCESS;
}

sp_status sp_mesh_box_hex_ids_rank(int32_t nx, int32_t ny, int32_t nz, int32_t p,
                                   uint64_t perm_seed, int32_t size, int32_t rank, int64_t* ids) {
  if (nx < 1 || ny < 1 || nz < 1 || p < 1 || !ids || size < 1 || rank < 0 || rank >= size)
    return fail(SP_ERR_INVALID_ARG, "sp_mesh_box_hex_ids_rank: bad arguments");
  const int64_t Nq = p + 1, Np = Nq * Nq * Nq, E = (int64_t)nx * ny * nz;
  if (E * Np > 2147483647LL)
    return fail(SP_ERR_SIZE, "sp_mesh_box_hex_ids_rank: %lld local nodes exceed int32",
                (long long)(E * Np));
  int sx, sy, sz;
  factor3(size, sx, sy, sz);
  std::vector<int32_t> rankAt((size_t)size);  // rank of grid cell cx + cy*sx + cz*sx*sy
  int rx = 0, ry = 0, rz = 0;
  for (int r = 0; r < size; ++r) {
    int a, b, c;
    rank_coords(sx, sy, sz, r, a, b, c);
    rankAt[(size_t)a + (size_t)b * sx + (size_t)c * sx * sy] = r;
    if (r == rank) {
      rx = a; ry = b; rz = c;
    }
  }
  // smallest local index on each point of one box's lattice (all boxes alike)
  const int64_t LX = (int64_t)nx * p + 1, LY = (int64_t)ny * p + 1, LZ = (int64_t)nz * p + 1;
  const std::vector<int32_t> slot = box_slots(E, perm_seed);
  std::vector<int32_t> minLocal((size_t)(LX * LY * LZ), 2147483647);
  for (int64_t e = 0; e < E; ++e) {
    const int64_t ex = e % nx, ey = (e / nx) % ny, ez = e / ((int64_t)nx * ny);
    for (int64_t k = 0; k < Nq; ++k)
      for (int64_t j = 0; j < Nq; ++j)
        for (int64_t i = 0; i < Nq; ++i) {
          const int64_t L = (ex * p + i) + (ey * p + j) * LX + (ez * p + k) * LX * LY;
          const int32_t l = (int32_t)((int64_t)slot[e] * Np + i + j * Nq + k * Nq * Nq);
          minLocal[L] = std::min(minLocal[L], l);
        }
  }
  // global lattice coordinate g (box extent w, boxes 0..s-1) -> the boxes holding it
  auto boxes = [](int64_t g, int64_t w, int s, int& lo, int& hi) {
    hi = (int)std::min<int64_t>(g / w, s - 1);
    lo = (g % w == 0 && g > 0) ? (int)(g / w) - 1 : hi;
  };
  for (int64_t e = 0; e < E; ++e) {
    const int64_t ex = e % nx, ey = (e / nx) % ny, ez = e / ((int64_t)nx * ny);
    const int64_t base = (int64_t)slot[e] * Np;
    for (int64_t k = 0; k < Nq; ++k)
      for (int64_t j = 0; j < Nq; ++j)
        for (int64_t i = 0; i < Nq; ++i) {
          const int64_t gx = (rx * (int64_t)nx + ex) * p + i;
          const int64_t gy = (ry * (int64_t)ny + ey) * p + j;
          const int64_t gz = (rz * (int64_t)nz + ez) * p + k;
          int x0, x1, y0, y1, z0, z1;
          boxes(gx, (int64_t)nx * p, sx, x0, x1);
          boxes(gy, (int64_t)ny * p, sy, y0, y1);
          boxes(gz, (int64_t)nz * p, sz, z0, z1);
          int best = size, bx = 0, by = 0, bz = 0;
          for (int cz = z0; cz <= z1; ++cz)
            for (int cy = y0; cy <= y1; ++cy)
              for (int cx = x0; cx <= x1; ++cx) {
                const int r = rankAt[(size_t)cx + (size_t)cy * sx + (size_t)cz * sx * sy];
                if (r < best) {
                  best = r; bx = cx; by = cy; bz = cz;
                }
              }
          const int64_t L = (gx - (int64_t)bx * nx * p) + (gy - (int64_t)by * ny * p) * LX +
                            (gz - (int64_t)bz * nz * p) * LX * LY;
          ids[base + i + j * Nq + k * Nq * Nq] = 1 + (int64_t)best * E * Np + minLocal[L];
        }
  }
  return SP_SUCCESS;
}

}  // extern "C"
