// Host check of the lane-row slab layout (build_slabs, compress_slabs) against the
// index arithmetic of kernel 7 (streamparanumal_gb300/csrc/sp_ogs_slab.cu), with no
// GPU: every slab's passes are walked as the kernel walks them -- full passes of KB
// members per lane at 32-word strides, the general row steps of a slab's rest, the
// any-size path, 16-bit member codes and row codes decoded through the slab's
// tables -- every index is checked against its array, and the gather and in-place
// gather+scatter they imply are compared bit for bit with the CSR-order sums.
//
// usage: slab_layout_check rs.bin ci.bin N order page_shift ball_shift seg_shift code_shift
//        [row_perm_seed]   (nonzero: the row words are a seeded permutation of the
//                           rows, as a renumbered walk folds its permutation in)
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <numeric>
#include <random>
#include <vector>

#include "sp_ogs_plan.h"

using namespace sp;

static long g_bad = 0;
#define CHECK(c, ...)                                   \
  do {                                                  \
    if (!(c)) {                                         \
      if (g_bad++ < 10) {                               \
        std::printf(__VA_ARGS__);                       \
        std::printf("\n");                              \
      }                                                 \
    }                                                   \
  } while (0)

static std::vector<int32_t> read_ints(const char* path) {
  FILE* f = std::fopen(path, "rb");
  if (!f) std::exit(3);
  std::fseek(f, 0, SEEK_END);
  const long n = std::ftell(f) / 4;
  std::fseek(f, 0, SEEK_SET);
  std::vector<int32_t> v(n);
  if (std::fread(v.data(), 4, n, f) != (size_t)n) std::exit(3);
  std::fclose(f);
  return v;
}

struct Layout {
  std::vector<int32_t> desc, ids, rows, tabs, td, rtabs, rtd;
  std::vector<uint16_t> codes, rcodes;
  int shift = 0;
};

// One member id of a full pass, as the kernel reads it (code decoded or id).
static int32_t member(const Layout& L, int64_t g, int64_t pos) {
  CHECK(pos >= 0 && pos < (int64_t)L.ids.size(), "id index %lld outside %zu", (long long)pos,
        L.ids.size());
  if (pos < 0 || pos >= (int64_t)L.ids.size()) return 0;
  if (L.shift > 0 && L.td[2 * g + 1] > 0) {
    const int32_t c = L.codes[pos], t = c >> L.shift;
    CHECK(t < L.td[2 * g + 1] && t < kSlabCodeTable, "table index %d of %d", t, L.td[2 * g + 1]);
    const int32_t col = L.tabs[L.td[2 * g] + t] | (c & ((1 << L.shift) - 1));
    CHECK(col == L.ids[pos], "code decodes to %d, id %d", col, L.ids[pos]);
    return col;
  }
  return L.ids[pos];
}

static int32_t row_word(const Layout& L, bool gather, int64_t pos) {
  if (!gather) return -1;
  CHECK(pos >= 0 && pos < (int64_t)L.rows.size(), "row word %lld outside %zu", (long long)pos,
        L.rows.size());
  return (pos >= 0 && pos < (int64_t)L.rows.size()) ? L.rows[pos] : 0;
}

// The row word of a full pass, as the kernel reads it: a row code decoded through
// the slab's row table (one word per lane) when the slab's rows compressed.
static int32_t pass_row_word(const Layout& L, bool gather, int64_t g, int64_t pos) {
  if (!gather || L.rtd.empty() || L.rtd[2 * g + 1] == 0) return row_word(L, gather, pos);
  CHECK(pos >= 0 && pos < (int64_t)L.rcodes.size(), "row code %lld outside %zu",
        (long long)pos, L.rcodes.size());
  if (pos < 0 || pos >= (int64_t)L.rcodes.size()) return 0;
  const int32_t c = L.rcodes[pos], t = c >> L.shift;
  CHECK(t < L.rtd[2 * g + 1] && L.rtd[2 * g + 1] <= kSlabRowTable, "row table index %d of %d", t,
        L.rtd[2 * g + 1]);
  const int64_t at = (int64_t)L.rtd[2 * g] + t;
  CHECK(at >= 0 && at < (int64_t)L.rtabs.size(), "row table word %lld", (long long)at);
  const int32_t r = L.rtabs[at] | (c & ((1 << L.shift) - 1));
  CHECK(r == L.rows[pos], "row code decodes to %d, row %d", r, L.rows[pos]);
  return r;
}

struct Sink {
  const std::vector<double>& q;
  std::vector<double>& gv;    // gather result
  std::vector<double>& out;   // in-place gather+scatter result
  bool gather;
  void row(int32_t r, const std::vector<int32_t>& cols) {
    double acc = 0.0;
    for (size_t t = 0; t < cols.size(); ++t) {
      CHECK(cols[t] >= 0 && cols[t] < (int32_t)q.size(), "column %d", cols[t]);
      acc = (t == 0) ? 0.0 + q[cols[t]] : acc + q[cols[t]];
    }
    if (gather) {
      CHECK(r >= 0 && r < (int32_t)gv.size(), "row %d", r);
      if (r >= 0 && r < (int32_t)gv.size()) gv[r] = acc;
    } else {
      for (int32_t c : cols) out[c] = acc;
    }
  }
};

static int pass_steps(int KB, int m) { return (m == 1 || m == 2 || m == 4 || m == 8) ? KB / m : 0; }

static void walk(const Layout& L, int KB, Sink& sink) {
  const int64_t nslabs = (int64_t)L.desc.size() / 4;
  for (int64_t g = 0; g < nslabs; ++g) {
    const int32_t E = L.desc[4 * g], rb = L.desc[4 * g + 1], m = L.desc[4 * g + 2];
    const int32_t w = L.desc[4 * g + 3];
    const int nl = w & 255, rem = (w >> 8) & 255, Re = w >> 16;
    CHECK(E % 4 == 0, "slab %lld starts off 16 bytes", (long long)g);
    CHECK(nl >= 1 && nl <= 32 && rem >= 1 && rem <= nl && Re >= 1, "descriptor %lld", (long long)g);
    const int P = pass_steps(KB, m);
    const int nfull = (nl == 32) ? (rem == 32 ? Re : Re - 1) : 0;
    int j0 = 0;
    if (P > 0) {
      for (; j0 + P <= nfull; j0 += P)  // full passes: member u of lane l at 32 u + l
        for (int lane = 0; lane < 32; ++lane) {
          const int64_t src = (int64_t)E + (int64_t)j0 * m * 32 + lane;
          for (int jj = 0; jj < P; ++jj) {
            std::vector<int32_t> cols;
            for (int t = 0; t < m; ++t) cols.push_back(member(L, g, src + 32 * (jj * m + t)));
            sink.row(pass_row_word(L, sink.gather, g, (int64_t)rb + (int64_t)(j0 + jj) * 32 + lane),
                     cols);
          }
        }
    }
    // the rest (and every slab of another size): one row step at a time, 32-bit ids
    for (int j = j0; j < Re; ++j) {
      const int wj = (j == Re - 1) ? rem : nl;
      for (int lane = 0; lane < wj; ++lane) {
        const int64_t src = (int64_t)E + (int64_t)j * m * nl + lane;
        std::vector<int32_t> cols;
        for (int t = 0; t < m; ++t) {
          const int64_t pos = src + (int64_t)t * wj;
          CHECK(pos < (int64_t)L.ids.size(), "id index %lld", (long long)pos);
          cols.push_back(pos < (int64_t)L.ids.size() ? L.ids[pos] : 0);
        }
        sink.row(row_word(L, sink.gather, (int64_t)rb + (int64_t)j * nl + lane), cols);
      }
    }
  }
}

int main(int argc, char** argv) {
  if (argc < 9) return 2;
  const auto rs = read_ints(argv[1]);
  const auto ci = read_ints(argv[2]);
  const int32_t N = std::atoi(argv[3]);
  const int order = std::atoi(argv[4]), page = std::atoi(argv[5]), ball = std::atoi(argv[6]);
  const int seg = std::atoi(argv[7]), shift = std::atoi(argv[8]);
  const unsigned row_seed = argc > 9 ? (unsigned)std::atoi(argv[9]) : 0u;
  const int32_t nrows = (int32_t)rs.size() - 1;
  std::vector<int32_t> pairs;
  if (!build_chunks(nrows, rs.data(), ci.data(), N, order, pairs, page, ball)) return 4;
  std::vector<int32_t> quads(pairs.size() * 2);
  for (size_t k = 0; k < pairs.size() / 2; ++k) {
    quads[4 * k] = pairs[2 * k];
    quads[4 * k + 1] = pairs[2 * k + 1];
    quads[4 * k + 2] = rs[pairs[2 * k]];
    quads[4 * k + 3] = rs[pairs[2 * k + 1]];
  }
  std::vector<double> q(N);
  std::mt19937_64 gen(7);
  for (auto& x : q) x = std::uniform_real_distribution<double>(-1.0, 1.0)(gen);
  std::vector<double> want_g(nrows), want_gs(q);
  for (int32_t r = 0; r < nrows; ++r) {
    double acc = 0.0;
    for (int32_t i = rs[r]; i < rs[r + 1]; ++i) acc = (i == rs[r]) ? 0.0 + q[ci[i]] : acc + q[ci[i]];
    want_g[r] = acc;
    for (int32_t i = rs[r]; i < rs[r + 1]; ++i) want_gs[ci[i]] = acc;
  }
  // row words: the rows themselves, or a seeded permutation of them
  std::vector<int32_t> perm(nrows);
  std::iota(perm.begin(), perm.end(), 0);
  if (row_seed) std::shuffle(perm.begin(), perm.end(), std::mt19937(row_seed));
  long coded = 0, total = 0, rows_coded = 0;
  for (int gather = 0; gather < 2; ++gather) {
    Layout L;
    build_slabs(quads, rs.data(), ci.data(), row_seed ? perm.data() : nullptr, seg, gather == 1,
                L.desc, L.ids, L.rows);
    if (shift > 0) {
      compress_slabs(L.desc, L.ids, shift, L.codes, L.tabs, L.td);
      L.shift = shift;
      if (gather) {
        compress_slab_rows(L.desc, L.rows, shift, L.rcodes, L.rtabs, L.rtd);
        for (size_t g = 0; g < L.desc.size() / 4; ++g) {
          const int32_t w = L.desc[4 * g + 3];
          if (L.rtd[2 * g + 1] > 0) rows_coded += ((w >> 16) - 1) * (w & 255) + ((w >> 8) & 255);
        }
      }
      for (size_t g = 0; g < L.desc.size() / 4; ++g) {
        const int32_t w = L.desc[4 * g + 3];
        const int64_t n = (int64_t)(((w >> 16) - 1) * (w & 255) + ((w >> 8) & 255)) * L.desc[4 * g + 2];
        total += n;
        if (L.td[2 * g + 1] > 0) coded += n;
      }
    }
    for (int KB : {8, 16}) {
      std::vector<double> gv(nrows, 7.0), out(q);
      Sink sink{q, gv, out, gather == 1};
      walk(L, KB, sink);
      if (gather) {
        for (int32_t r = 0; r < nrows; ++r)
          CHECK(std::memcmp(&gv[perm[r]], &want_g[r], 8) == 0 ||
                    (rs[r] == rs[r + 1] && gv[perm[r]] == 0.0),
                "gather row %d differs (KB %d)", r, KB);
      } else {
        CHECK(std::memcmp(out.data(), want_gs.data(), 8 * out.size()) == 0,
              "gather+scatter differs (KB %d)", KB);
      }
    }
  }
  std::printf("%s coded %ld of %ld rows %ld of %d\n", g_bad ? "FAILED" : "ok", coded, total,
              rows_coded, nrows);
  return g_bad ? 1 : 0;
}
