// Host-side construction of gather-scatter plans from global ids, and the
// structured hex box id generator.  Runs once per mesh, outside timed regions.
//
// Grouping rules (ogsBase_t::Setup, libs/ogs/ogsSetup.cpp:87-290, at one rank):
//   * entries with id 0 are ignored; the rest are grouped by |id|;
//   * with `unique`, every group gets exactly one positive member, chosen with the
//     reference's LCG stream (libs/primitives/random.cpp:47-172, seeded with the
//     rank at Setup, ogsSetup.cpp:110): group n (groups in ascending |id|) keeps
//     member rand[n] % size positive.  Members are taken in ascending local index;
//     the reference takes them in the order of an unstable sort, so the chosen
//     owner can differ -- Sym and Trans results do not depend on it;
//   * rows: groups with a positive member first, each class in order of first
//     appearance of its smallest local index (EnumerateGatherGroups,
//     ogsSetup.cpp:492-559);
//   * columns inside a row ascend by local index (stable SortByRow, :561-579);
//   * the N operator keeps the positive members (Signed kind); for Unsigned it is T.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#include "sp_ogs_plan.h"

namespace sp {

static inline int64_t iabs64(int64_t v) { return v < 0 ? -v : v; }

// Groups of |id| as (key, member list ascending local index), keys ascending.
struct Groups {
  std::vector<int32_t> offsets;  // ngroups + 1
  std::vector<int32_t> members;  // local indices, grouped
};

static void build_groups(int32_t N, const int64_t* ids, Groups& g) {
  int64_t maxAbs = 0;
  int32_t nids = 0;
#pragma omp parallel for schedule(static) reduction(max : maxAbs) reduction(+ : nids)
  for (int32_t l = 0; l < N; ++l)
    if (ids[l] != 0) {
      maxAbs = std::max(maxAbs, iabs64(ids[l]));
      ++nids;
    }
  g.offsets.assign(1, 0);
  g.members.clear();
  if (nids == 0) return;
  const int64_t directLimit = std::max<int64_t>(4 * (int64_t)N, 1 << 20);
  if (maxAbs <= directLimit) {
    // counting sort by key, in parallel: histogram, scan, atomic placement, then
    // each group's members sorted (groups are small), so the result is the stable
    // order whatever the thread schedule
    const size_t nkeys = (size_t)maxAbs + 2;
    std::vector<int32_t> cnt(nkeys, 0);
#pragma omp parallel for schedule(static)
    for (int32_t l = 0; l < N; ++l)
      if (ids[l] != 0) {
#pragma omp atomic
        ++cnt[(size_t)iabs64(ids[l]) + 1];
      }
    std::vector<int32_t> fill(nkeys, 0);
    int32_t running = 0;
    for (size_t k = 1; k < nkeys; ++k) {
      if (cnt[k] != 0) g.offsets.push_back(running + cnt[k]);
      running += cnt[k];
      fill[k - 1] = running - cnt[k];  // start of key k-1's bucket
    }
    g.members.resize(nids);
#pragma omp parallel for schedule(static)
    for (int32_t l = 0; l < N; ++l)
      if (ids[l] != 0) {
        int32_t pos;
#pragma omp atomic capture
        pos = fill[(size_t)iabs64(ids[l])]++;
        g.members[pos] = l;
      }
    const int32_t ng = (int32_t)g.offsets.size() - 1;
#pragma omp parallel for schedule(dynamic, 4096)
    for (int32_t n = 0; n < ng; ++n)
      std::sort(g.members.begin() + g.offsets[n], g.members.begin() + g.offsets[n + 1]);
  } else {
    std::vector<std::pair<int64_t, int32_t>> kv;
    kv.reserve(nids);
    for (int32_t l = 0; l < N; ++l)
      if (ids[l] != 0) kv.emplace_back(iabs64(ids[l]), l);
    std::sort(kv.begin(), kv.end());
    g.members.resize(nids);
    for (int32_t i = 0; i < nids; ++i) {
      g.members[i] = kv[i].second;
      if (i > 0 && kv[i].first != kv[i - 1].first) g.offsets.push_back(i);
    }
    g.offsets.push_back(nids);
  }
}

// Element slots of a box (lexicographic element e = ex + ey*nx + ez*nx*ny is stored
// at slot[e]): the identity, or a Fisher-Yates shuffle driven by SplitMix64 from
// perm_seed.
std::vector<int32_t> box_slots(int64_t E, uint64_t perm_seed) {
  std::vector<int32_t> slot(E);
  std::iota(slot.begin(), slot.end(), 0);
  if (perm_seed != 0) {
    uint64_t st = perm_seed;
    auto splitmix = [&st]() {
      uint64_t z = (st += 0x9E3779B97F4A7C15ULL);
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
      return z ^ (z >> 31);
    };
    for (int64_t i = E - 1; i > 0; --i) {
      const int64_t j = (int64_t)(splitmix() % (uint64_t)(i + 1));
      std::swap(slot[i], slot[j]);
    }
  }
  return slot;
}

}  // namespace sp

using namespace sp;

extern "C" {

sp_status sp_ogs_setup_csr(int32_t N, int64_t* ids, sp_kind kind, int32_t unique,
                           int32_t* NrowsT, int32_t* rowStartsT, int32_t* colIdsT,
                           int32_t* NrowsN, int32_t* rowStartsN, int32_t* colIdsN) {
  if (N < 0 || (N > 0 && !ids)) return fail(SP_ERR_INVALID_ARG, "sp_ogs_setup_csr: bad ids");
  if (!NrowsT || !rowStartsT || !NrowsN || !rowStartsN || (N > 0 && (!colIdsT || !colIdsN)))
    return fail(SP_ERR_INVALID_ARG, "sp_ogs_setup_csr: null output array");
  if (kind < SP_KIND_UNSIGNED || kind > SP_KIND_HALO)
    return fail(SP_ERR_INVALID_ARG, "sp_ogs_setup_csr: bad kind");
  if ((kind == SP_KIND_UNSIGNED && unique) || (kind == SP_KIND_HALO && unique))
    return fail(SP_ERR_INVALID_ARG, "Invalid ogs setup requested");

  Groups g;
  build_groups(N, ids, g);
  const int32_t ngroups = (int32_t)g.offsets.size() - 1;

  if (unique) {
    // the draws follow the groups in ascending |id| (one sequential LCG pass), the
    // sign writes are independent per group
    std::vector<int32_t> draw(ngroups);
    Lcg rng(0);  // seedRNG(rank) with rank 0
    for (int32_t n = 0; n < ngroups; ++n) draw[n] = rng.next_int();
#pragma omp parallel for schedule(static)
    for (int32_t n = 0; n < ngroups; ++n) {
      const int32_t a = g.offsets[n], b = g.offsets[n + 1];
      const int32_t m = draw[n] % (b - a);
      const int64_t key = iabs64(ids[g.members[a]]);
      for (int32_t i = a; i < b; ++i) ids[g.members[i]] = -key;
      if (m >= 0) ids[g.members[a + m]] = key;
    }
  }

  // group sign; members ascend, so members[offsets[n]] is the first appearance
  std::vector<uint8_t> positive(ngroups, 0);
  std::vector<int32_t> firstOf(N > 0 ? N : 1, -1);
#pragma omp parallel for schedule(static)
  for (int32_t n = 0; n < ngroups; ++n) {
    for (int32_t i = g.offsets[n]; i < g.offsets[n + 1]; ++i)
      if (ids[g.members[i]] > 0) {
        positive[n] = 1;
        break;
      }
    firstOf[g.members[g.offsets[n]]] = n;
  }
  // rows: positive groups by first appearance, then the flagged-only groups.  A
  // group's first member is its smallest local index, so scanning local indices in
  // ascending order meets the groups in first-appearance order (linear time).
  std::vector<int32_t> order;
  order.reserve(ngroups);
  for (int pass = 1; pass >= 0; --pass)
    for (int32_t l = 0; l < N; ++l) {
      const int32_t n = firstOf[l];
      if (n >= 0 && positive[n] == pass) order.push_back(n);
    }
  std::vector<int32_t>().swap(firstOf);
  int32_t NrowsP = 0;
  for (int32_t n = 0; n < ngroups; ++n) NrowsP += positive[n];

  *NrowsT = ngroups;
  rowStartsT[0] = 0;
  for (int32_t r = 0; r < ngroups; ++r) {
    const int32_t n = order[r];
    rowStartsT[r + 1] = rowStartsT[r] + (g.offsets[n + 1] - g.offsets[n]);
  }
#pragma omp parallel for schedule(static)
  for (int32_t r = 0; r < ngroups; ++r) {
    const int32_t n = order[r];
    std::copy(g.members.begin() + g.offsets[n], g.members.begin() + g.offsets[n + 1],
              colIdsT + rowStartsT[r]);
  }
  // N operator: positive members (Signed, Halo) or every member (Unsigned)
  *NrowsN = NrowsP;
  std::vector<int32_t> cntN(NrowsP + 1, 0);
#pragma omp parallel for schedule(static)
  for (int32_t r = 0; r < NrowsP; ++r) {
    int32_t c = 0;
    for (int32_t i = rowStartsT[r]; i < rowStartsT[r + 1]; ++i)
      c += (kind == SP_KIND_UNSIGNED || ids[colIdsT[i]] > 0) ? 1 : 0;
    cntN[r] = c;
  }
  rowStartsN[0] = 0;
  for (int32_t r = 0; r < NrowsP; ++r) rowStartsN[r + 1] = rowStartsN[r] + cntN[r];
#pragma omp parallel for schedule(static)
  for (int32_t r = 0; r < NrowsP; ++r) {
    int32_t nn = rowStartsN[r];
    for (int32_t i = rowStartsT[r]; i < rowStartsT[r + 1]; ++i)
      if (kind == SP_KIND_UNSIGNED || ids[colIdsT[i]] > 0) colIdsN[nn++] = colIdsT[i];
  }
  return SP_SUCCESS;
}

sp_status sp_ogs_setup(int32_t N, int64_t* ids, sp_kind kind, int32_t unique, sp_stream_t stream,
                       sp_ogs_plan** out) {
  if (!out) return fail(SP_ERR_INVALID_ARG, "sp_ogs_setup: null out");
  *out = nullptr;
  if (N < 0) return fail(SP_ERR_INVALID_ARG, "sp_ogs_setup: negative N");
  std::vector<int32_t> rsT(N + 1), ciT(std::max(N, 1)), rsN(N + 1), ciN(std::max(N, 1));
  int32_t NrowsT = 0, NrowsN = 0;
  sp_status st = sp_ogs_setup_csr(N, ids, kind, unique, &NrowsT, rsT.data(), ciT.data(), &NrowsN,
                                  rsN.data(), ciN.data());
  if (st) return st;
  if (kind == SP_KIND_UNSIGNED)  // N shares T's CSR over its first NrowsN rows
    return sp_ogs_plan_create(N, NrowsT, rsT.data(), ciT.data(), NrowsN, nullptr, nullptr, stream,
                              out);
  return sp_ogs_plan_create(N, NrowsT, rsT.data(), ciT.data(), NrowsN, rsN.data(), ciN.data(),
                            stream, out);
}

sp_status sp_mesh_box_hex_ids(int32_t nx, int32_t ny, int32_t nz, int32_t p, uint64_t perm_seed,
                              int64_t* ids) {
  if (nx < 1 || ny < 1 || nz < 1 || p < 1 || !ids)
    return fail(SP_ERR_INVALID_ARG, "sp_mesh_box_hex_ids: bad arguments");
  const int64_t Nq = p + 1, Np = Nq * Nq * Nq;
  const int64_t E = (int64_t)nx * ny * nz;
  const int64_t Ntot = E * Np;
  if (Ntot > 2147483647LL)
    return fail(SP_ERR_SIZE, "sp_mesh_box_hex_ids: %lld local nodes exceed int32", (long long)Ntot);
  const int64_t LX = (int64_t)nx * p + 1, LY = (int64_t)ny * p + 1, LZ = (int64_t)nz * p + 1;

  const std::vector<int32_t> slot = box_slots(E, perm_seed);
  // smallest local index on each lattice point
  std::vector<int32_t> minLocal((size_t)(LX * LY * LZ), 2147483647);
  for (int64_t e = 0; e < E; ++e) {
    const int64_t ex = e % nx, ey = (e / nx) % ny, ez = e / ((int64_t)nx * ny);
    const int64_t base = (int64_t)slot[e] * Np;
    for (int64_t k = 0; k < Nq; ++k)
      for (int64_t j = 0; j < Nq; ++j)
        for (int64_t i = 0; i < Nq; ++i) {
          const int64_t L = (ex * p + i) + (ey * p + j) * LX + (ez * p + k) * LX * LY;
          const int32_t l = (int32_t)(base + i + j * Nq + k * Nq * Nq);
          if (l < minLocal[L]) minLocal[L] = l;
        }
  }
  for (int64_t e = 0; e < E; ++e) {
    const int64_t ex = e % nx, ey = (e / nx) % ny, ez = e / ((int64_t)nx * ny);
    const int64_t base = (int64_t)slot[e] * Np;
    for (int64_t k = 0; k < Nq; ++k)
      for (int64_t j = 0; j < Nq; ++j)
        for (int64_t i = 0; i < Nq; ++i) {
          const int64_t L = (ex * p + i) + (ey * p + j) * LX + (ez * p + k) * LX * LY;
          ids[base + i + j * Nq + k * Nq * Nq] = 1 + (int64_t)minLocal[L];
        }
  }
  return SP_SUCCESS;
}

}  // extern "C"
