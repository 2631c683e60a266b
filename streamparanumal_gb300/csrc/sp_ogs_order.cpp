// Warp chunks of a gather-scatter operator and the order they are scheduled in.
//
// A chunk is a contiguous row range [r0, r1) holding at most kWarpChunkNnz
// non-zeros; one warp processes one chunk.  Any partition of the rows gives the
// same results (each row is summed by one lane in CSR order), so the partition and
// the chunk order are free to serve memory locality:
//   order 0 (natural): chunks follow the row order;
//   order 1 (bfs): rows are grouped by the page (2^page_shift entries of local data,
//     knob ogs.page_shift) holding their first member, pages are visited
//     breadth-first over the "row joins pages" graph, and each page's rows are cut
//     into chunks in that order.  Pages that share rows are then processed close
//     together in time, so the data one chunk touches in a neighbouring page is
//     usually still in L2 when that page's own chunks run -- whatever the element
//     numbering in memory.  A page of about one element's nodes makes the visit a
//     wavefront over the mesh.  With ball_shift > 0 the pages are visited as a
//     chain of breadth-first balls of 2^ball_shift entries instead (page_order).
#include <parallel/algorithm>

#include <algorithm>
#include <cstdint>
#include <utility>
#include <vector>

#include "sp_ogs_plan.h"

namespace sp {

static void cut_run(int32_t ra, int32_t rb, const int32_t* rs, std::vector<int32_t>& chunks) {
  int32_t c0 = ra;
  for (int32_t r = ra; r < rb; ++r) {
    if (rs[r + 1] - rs[c0] > kWarpChunkNnz || r - c0 >= kWarpChunkNnz) {
      chunks.push_back(c0);
      chunks.push_back(r);
      c0 = r;
    }
  }
  if (rb > c0) {
    chunks.push_back(c0);
    chunks.push_back(rb);
  }
}

// Number of chunks cut_run makes of rows [ra, rb).
static int32_t count_run(int32_t ra, int32_t rb, const int32_t* rs) {
  int32_t n = 0, c0 = ra;
  for (int32_t r = ra; r < rb; ++r)
    if (rs[r + 1] - rs[c0] > kWarpChunkNnz || r - c0 >= kWarpChunkNnz) {
      ++n;
      c0 = r;
    }
  return n + (rb > c0 ? 1 : 0);
}

// Calls f(ra, rb) for each maximal run of consecutive rows in rows[a, b).
template <typename F>
static void for_runs(const int32_t* rows, int32_t a, int32_t b, F f) {
  int32_t k = a;
  while (k < b) {
    const int32_t ra = rows[k];
    int32_t rb = ra + 1;
    ++k;
    while (k < b && rows[k] == rb) {
      ++rb;
      ++k;
    }
    f(ra, rb);
  }
}

// Pages of local data (2^page_shift entries) visited breadth-first over the "row
// joins pages" graph, restarting at the lowest unvisited page.
struct PageOrder {
  int32_t npages = 0, nonEmpty = 0;
  std::vector<int32_t> rowPage;   // page of each row's first member, -1 if empty
  std::vector<int32_t> pageRows;  // rows grouped by page, ascending inside
  std::vector<int32_t> pstart;    // rows of page p: pageRows[pstart[p], pstart[p+1])
  std::vector<int32_t> queue;     // pages in visit order
};

static void page_order(int32_t nrows, const int32_t* rs, const int32_t* ci, int32_t ncols,
                       int page_shift, int ball_shift, PageOrder& po) {
  const int64_t npages64 = ((int64_t)std::max(ncols, 1) + (1LL << page_shift) - 1) >> page_shift;
  const int32_t npages = (int32_t)npages64;
  po.npages = npages;
  // page of each row's first member, and the rows grouped by page (ascending row
  // inside).  Rows numbered by first appearance have non-decreasing pages, which
  // makes the grouping a pass over the rows; otherwise (page, row) keys are sorted.
  std::vector<int32_t>& rowPage = po.rowPage;
  rowPage.assign(nrows, -1);
  int32_t unordered = 0, nonEmpty = 0;
#pragma omp parallel for schedule(static) reduction(+ : nonEmpty)
  for (int32_t r = 0; r < nrows; ++r)
    if (rs[r + 1] > rs[r]) {
      rowPage[r] = ci[rs[r]] >> page_shift;
      ++nonEmpty;
    }
#pragma omp parallel for schedule(static) reduction(max : unordered)
  for (int32_t r = 1; r < nrows; ++r)
    if (rowPage[r] < 0 || rowPage[r - 1] < 0 || rowPage[r] < rowPage[r - 1]) unordered = 1;
  po.nonEmpty = nonEmpty;
  std::vector<int32_t>& pageRows = po.pageRows;
  pageRows.assign(nonEmpty, 0);
  std::vector<int32_t>& pstart = po.pstart;
  pstart.assign(npages + 1, 0);
  if (!unordered) {
#pragma omp parallel for schedule(static)
    for (int32_t r = 0; r < nrows; ++r) {
      pageRows[r] = r;
      if (r == 0 || rowPage[r] != rowPage[r - 1])
        for (int32_t q = (r == 0 ? 0 : rowPage[r - 1] + 1); q <= rowPage[r]; ++q) pstart[q] = r;
    }
    for (int32_t q = rowPage[nrows - 1] + 1; q <= npages; ++q) pstart[q] = nrows;
  } else {
    std::vector<int64_t> key;
    key.reserve(nonEmpty);
    for (int32_t r = 0; r < nrows; ++r)
      if (rowPage[r] >= 0) key.push_back(((int64_t)rowPage[r] << 32) | r);
    __gnu_parallel::sort(key.begin(), key.end());
    std::vector<int32_t> pcount(npages + 1, 0);
    for (int32_t k = 0; k < nonEmpty; ++k) {
      pageRows[k] = (int32_t)(key[k] & 0xffffffff);
      ++pcount[(int32_t)(key[k] >> 32) + 1];
    }
    for (int32_t q = 0; q < npages; ++q) pstart[q + 1] = pstart[q] + pcount[q + 1];
  }
  // forward edges (a row's first page -> the pages of its other members), unique per
  // page: counted, then written
  auto forward = [&](int32_t p, std::vector<int32_t>& tmp) {
    tmp.clear();
    for (int32_t k = pstart[p]; k < pstart[p + 1]; ++k) {
      const int32_t r = pageRows[k];
      for (int32_t i = rs[r] + 1; i < rs[r + 1]; ++i) {
        const int32_t q = ci[i] >> page_shift;
        if (q != p) tmp.push_back(q);
      }
    }
    std::sort(tmp.begin(), tmp.end());
    tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
  };
  std::vector<int64_t> fstart(npages + 1, 0);
#pragma omp parallel
  {
    std::vector<int32_t> tmp;
#pragma omp for schedule(dynamic, 1024)
    for (int32_t p = 0; p < npages; ++p) {
      forward(p, tmp);
      fstart[p + 1] = (int64_t)tmp.size();
    }
  }
  for (int32_t p = 0; p < npages; ++p) fstart[p + 1] += fstart[p];
  std::vector<int32_t> fwd(fstart[npages]);
#pragma omp parallel
  {
    std::vector<int32_t> tmp;
#pragma omp for schedule(dynamic, 1024)
    for (int32_t p = 0; p < npages; ++p) {
      forward(p, tmp);
      std::copy(tmp.begin(), tmp.end(), fwd.begin() + fstart[p]);
    }
  }
  // undirected adjacency: forward lists plus their reverses, sorted and unique
  std::vector<int64_t> adjStart(npages + 1, 0);
  {
    std::vector<int32_t> rev(npages, 0);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < fstart[npages]; ++e) {
#pragma omp atomic
      ++rev[fwd[e]];
    }
    for (int32_t p = 0; p < npages; ++p)
      adjStart[p + 1] = adjStart[p] + (fstart[p + 1] - fstart[p]) + rev[p];
  }
  std::vector<int32_t> adj(adjStart[npages]);
  std::vector<int64_t> fill(npages);
#pragma omp parallel for schedule(static)
  for (int32_t p = 0; p < npages; ++p) {
    std::copy(fwd.begin() + fstart[p], fwd.begin() + fstart[p + 1], adj.begin() + adjStart[p]);
    fill[p] = adjStart[p] + (fstart[p + 1] - fstart[p]);
  }
#pragma omp parallel for schedule(dynamic, 1024)
  for (int32_t p = 0; p < npages; ++p)
    for (int64_t e = fstart[p]; e < fstart[p + 1]; ++e) {
      const int32_t q = fwd[e];
      int64_t at;
#pragma omp atomic capture
      at = fill[q]++;
      adj[at] = p;
    }
  std::vector<int64_t> adjEnd(npages);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int32_t p = 0; p < npages; ++p) {
    int32_t* b = adj.data() + adjStart[p];
    int32_t* e = adj.data() + adjStart[p + 1];
    std::sort(b, e);
    adjEnd[p] = std::unique(b, e) - adj.data();
  }
  std::vector<uint8_t> seen(npages, 0);
  std::vector<int32_t>& queue = po.queue;
  queue.clear();
  queue.reserve(npages);
  if (ball_shift > 0) {
    // balls: breadth-first from a seed until the ball holds 2^ball_shift entries,
    // each next seed an unvisited neighbour of the most recent ball's rim (else the
    // lowest unvisited page).  The walk then moves through the mesh as a chain of
    // compact regions, so a page's neighbours are visited within a few balls of it
    // instead of one breadth-first shell (a whole cross-section of the mesh) away.
    const int64_t cap = std::max<int64_t>(1, (int64_t)1 << std::max(0, ball_shift - page_shift));
    std::vector<int32_t> rim;  // pages of finished balls whose neighbours were not all taken
    int32_t low = 0;
    while ((int64_t)queue.size() < npages) {
      int32_t seed = -1;
      while (seed < 0 && !rim.empty()) {
        const int32_t p = rim.back();
        bool open = false;
        for (int64_t k = adjStart[p]; k < adjEnd[p] && seed < 0; ++k)
          if (!seen[adj[k]]) seed = adj[k];
        for (int64_t k = adjStart[p]; k < adjEnd[p] && !open; ++k)
          if (!seen[adj[k]] && adj[k] != seed) open = true;
        if (!open) rim.pop_back();
      }
      if (seed < 0) {
        while (seen[low]) ++low;
        seed = low;
      }
      const size_t b0 = queue.size();
      seen[seed] = 1;
      queue.push_back(seed);
      size_t head = b0;
      while (head < queue.size() && (int64_t)(queue.size() - b0) < cap) {
        const int32_t p = queue[head++];
        for (int64_t k = adjStart[p]; k < adjEnd[p] && (int64_t)(queue.size() - b0) < cap; ++k) {
          const int32_t q = adj[k];
          if (!seen[q]) {
            seen[q] = 1;
            queue.push_back(q);
          }
        }
      }
      // the ball's rim: pages whose neighbours may still be unvisited
      for (size_t k = (head > b0 ? head - 1 : b0); k < queue.size(); ++k) rim.push_back(queue[k]);
    }
    return;
  }
  // breadth-first page order, restarting at the lowest unvisited page
  for (int32_t start = 0; start < npages; ++start) {
    if (seen[start]) continue;
    seen[start] = 1;
    size_t head = queue.size();
    queue.push_back(start);
    while (head < queue.size()) {
      const int32_t p = queue[head++];
      for (int64_t k = adjStart[p]; k < adjEnd[p]; ++k) {
        const int32_t q = adj[k];
        if (!seen[q]) {
          seen[q] = 1;
          queue.push_back(q);
        }
      }
    }
  }
}

bool build_chunks(int32_t nrows, const int32_t* rs, const int32_t* ci, int32_t ncols, int order,
                  std::vector<int32_t>& chunks, int page_shift, int ball_shift,
                  std::vector<int32_t>* pages) {
  chunks.clear();
  int32_t tooBig = 0;
#pragma omp parallel for schedule(static) reduction(max : tooBig)
  for (int32_t r = 0; r < nrows; ++r)
    if (rs[r + 1] - rs[r] > kWarpChunkNnz) tooBig = 1;
  if (tooBig) return false;
  if (nrows == 0) return true;
  if (order == 0) {
    cut_run(0, nrows, rs, chunks);
    return true;
  }
  PageOrder po;
  page_order(nrows, rs, ci, ncols, page_shift, ball_shift, po);
  if (pages) *pages = po.queue;
  const int32_t npages = po.npages, nonEmpty = po.nonEmpty;
  const std::vector<int32_t>& rowPage = po.rowPage;
  const std::vector<int32_t>& pageRows = po.pageRows;
  const std::vector<int32_t>& pstart = po.pstart;
  const std::vector<int32_t>& queue = po.queue;
  // chunks: each page's rows as maximal consecutive runs, pages in visit order;
  // counted per page, then cut in parallel into their places
  std::vector<int64_t> cstart(npages + 1, 0);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int32_t k = 0; k < npages; ++k) {
    const int32_t p = queue[k];
    int64_t n = 0;
    for_runs(pageRows.data(), pstart[p], pstart[p + 1],
             [&](int32_t ra, int32_t rb) { n += count_run(ra, rb, rs); });
    cstart[k + 1] = n;
  }
  for (int32_t k = 0; k < npages; ++k) cstart[k + 1] += cstart[k];
  const int32_t nEmpty = nrows - nonEmpty;
  chunks.resize(2 * (cstart[npages] + nEmpty));
#pragma omp parallel
  {
    std::vector<int32_t> tmp;
#pragma omp for schedule(dynamic, 1024)
    for (int32_t k = 0; k < npages; ++k) {
      const int32_t p = queue[k];
      tmp.clear();
      for_runs(pageRows.data(), pstart[p], pstart[p + 1],
               [&](int32_t ra, int32_t rb) { cut_run(ra, rb, rs, tmp); });
      std::copy(tmp.begin(), tmp.end(), chunks.begin() + 2 * cstart[k]);
    }
  }
  // rows without members (possible in a caller-built CSR) still need a chunk
  int64_t at = 2 * cstart[npages];
  for (int32_t r = 0; r < nrows && nEmpty > 0; ++r)
    if (rowPage[r] < 0) {
      chunks[at++] = r;
      chunks[at++] = r + 1;
    }
  return true;
}

void bfs_row_sequence(int32_t nrows, const int32_t* rs, const int32_t* ci, int32_t ncols,
                      int page_shift, int ball_shift, std::vector<int32_t>& seq,
                      std::vector<int32_t>* pages) {
  seq.clear();
  if (nrows == 0) return;
  PageOrder po;
  page_order(nrows, rs, ci, ncols, page_shift, ball_shift, po);
  if (pages) *pages = po.queue;
  seq.resize(nrows);
  std::vector<int64_t> at(po.npages + 1, 0);
  for (int32_t k = 0; k < po.npages; ++k) {
    const int32_t p = po.queue[k];
    at[k + 1] = at[k] + (po.pstart[p + 1] - po.pstart[p]);
  }
#pragma omp parallel for schedule(dynamic, 1024)
  for (int32_t k = 0; k < po.npages; ++k) {
    const int32_t p = po.queue[k];
    std::copy(po.pageRows.begin() + po.pstart[p], po.pageRows.begin() + po.pstart[p + 1],
              seq.begin() + at[k]);
  }
  int64_t n = at[po.npages];
  for (int32_t r = 0; r < nrows && n < nrows; ++r)
    if (po.rowPage[r] < 0) seq[n++] = r;
}

void build_grouped(const std::vector<int32_t>& quads, int32_t nrows, const int32_t* rs,
                   const int32_t* ci, std::vector<int32_t>& rowsG, std::vector<int32_t>& ciG) {
  const int64_t nchunks = (int64_t)quads.size() / 4;
  rowsG.assign(nrows, 0);
  ciG.assign(nrows > 0 ? rs[nrows] : 0, 0);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t c = 0; c < nchunks; ++c) {
    const int32_t r0 = quads[4 * c], r1 = quads[4 * c + 1], g0 = quads[4 * c + 2];
    int32_t order[kWarpChunkNnz];
    const int32_t nr = r1 - r0;
    for (int32_t k = 0; k < nr; ++k) order[k] = k;
    std::stable_sort(order, order + nr, [&](int32_t a, int32_t b) {
      return rs[r0 + a + 1] - rs[r0 + a] > rs[r0 + b + 1] - rs[r0 + b];
    });
    int32_t at = g0;
    for (int32_t k = 0; k < nr; ++k) {
      const int32_t r = r0 + order[k];
      rowsG[r0 + k] = (at - g0) | (order[k] << 16);
      for (int32_t i = rs[r]; i < rs[r + 1]; ++i) ciG[at++] = ci[i];
    }
  }
}

void build_sorted(const std::vector<int32_t>& quads, int32_t nrows, const int32_t* rs,
                  const int32_t* rowsG, const int32_t* ciE, std::vector<int32_t>& colS,
                  std::vector<uint8_t>& rowOf, std::vector<uint8_t>& e2s) {
  const int64_t nchunks = (int64_t)quads.size() / 4;
  const int32_t nnz = nrows > 0 ? rs[nrows] : 0;
  colS.assign(nnz, 0);
  rowOf.assign(nnz, 0);
  e2s.assign(nnz, 0);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t c = 0; c < nchunks; ++c) {
    const int32_t r0 = quads[4 * c], r1 = quads[4 * c + 1], g0 = quads[4 * c + 2];
    const int32_t n = quads[4 * c + 3] - g0, nr = r1 - r0;
    uint8_t rowOfE[kWarpChunkNnz];  // row offset of each entry of the row walk
    if (rowsG) {
      for (int32_t k = 0; k < nr; ++k) {
        const int32_t a = rowsG[r0 + k] & 0xFFFF;
        const int32_t b = (k + 1 < nr) ? (rowsG[r0 + k + 1] & 0xFFFF) : n;
        for (int32_t e = a; e < b; ++e) rowOfE[e] = (uint8_t)(rowsG[r0 + k] >> 16);
      }
    } else {
      for (int32_t r = r0; r < r1; ++r)
        for (int32_t i = rs[r]; i < rs[r + 1]; ++i) rowOfE[i - g0] = (uint8_t)(r - r0);
    }
    // column << 8 | entry: sorts by column (every column appears once in a chunk)
    int64_t key[kWarpChunkNnz];
    for (int32_t e = 0; e < n; ++e) key[e] = ((int64_t)ciE[g0 + e] << 8) | e;
    std::sort(key, key + n);
    for (int32_t j = 0; j < n; ++j) {
      const int32_t e = (int32_t)(key[j] & 0xFF);
      colS[g0 + j] = (int32_t)(key[j] >> 8);
      rowOf[g0 + j] = rowOfE[e];
      e2s[g0 + e] = (uint8_t)j;
    }
  }
}

// Rows of chunks [c0, c1) in their walk order, stably regrouped by member count,
// largest first (rows without members last, and only when `with_empty`).
static void segment_rows(const std::vector<int32_t>& quads, int64_t c0, int64_t c1,
                         const int32_t* rs, bool with_empty, std::vector<int64_t>& key) {
  key.clear();
  for (int64_t c = c0; c < c1; ++c)
    for (int32_t r = quads[4 * c]; r < quads[4 * c + 1]; ++r) {
      const int64_t m = rs[r + 1] - rs[r];
      if (m > 0 || with_empty) key.push_back(((int64_t)(kOgsMaxRowSize - m) << 32) | (uint32_t)r);
    }
  std::stable_sort(key.begin(), key.end(),
                   [](int64_t a, int64_t b) { return (a >> 32) < (b >> 32); });
}

// Words a slab of `entries` ids occupies: rounded up to 16 bytes, so that every
// slab, and every pass of whole row steps inside it, starts on a 16-byte boundary.
static inline int64_t slab_span(int64_t entries) { return (entries + 3) & ~int64_t(3); }

int32_t slab_rows_per_lane(int32_t m) {
  if (m <= 0) return kSlabLaneEntries;
  return m <= kSlabLaneEntries ? kSlabLaneEntries / m : 1;
}

void build_slabs(const std::vector<int32_t>& quads, const int32_t* rs, const int32_t* ci,
                 const int32_t* perm, int seg_shift, bool with_rows, std::vector<int32_t>& desc,
                 std::vector<int32_t>& ids, std::vector<int32_t>& rows) {
  const int64_t nchunks = (int64_t)quads.size() / 4;
  // segments: runs of consecutive chunks of the walk holding >= 2^seg_shift entries
  std::vector<int64_t> seg{0};
  int64_t acc = 0;
  for (int64_t c = 0; c < nchunks; ++c) {
    acc += quads[4 * c + 3] - quads[4 * c + 2];
    if (acc >= (int64_t(1) << seg_shift)) {
      seg.push_back(c + 1);
      acc = 0;
    }
  }
  if (seg.back() != nchunks) seg.push_back(nchunks);
  const int64_t nseg = (int64_t)seg.size() - 1;
  // pass 1: slabs, entries and rows of every segment
  std::vector<int64_t> nS(nseg + 1, 0), nE(nseg + 1, 0), nW(nseg + 1, 0);
#pragma omp parallel
  {
    std::vector<int64_t> key;
#pragma omp for schedule(dynamic, 16)
    for (int64_t g = 0; g < nseg; ++g) {
      segment_rows(quads, seg[g], seg[g + 1], rs, with_rows, key);
      int64_t S = 0, E = 0;
      for (size_t a = 0; a < key.size();) {
        const int32_t m = kOgsMaxRowSize - (int32_t)(key[a] >> 32);
        size_t b = a;
        while (b < key.size() && (key[b] >> 32) == (key[a] >> 32)) ++b;
        const int64_t cap = 32LL * slab_rows_per_lane(m);
        for (int64_t k0 = (int64_t)a; k0 < (int64_t)b; k0 += cap) {
          ++S;
          E += slab_span(std::min<int64_t>(cap, (int64_t)b - k0) * m);
        }
        a = b;
      }
      nS[g + 1] = S;
      nE[g + 1] = E;
      nW[g + 1] = with_rows ? (int64_t)key.size() : 0;
    }
  }
  for (int64_t g = 0; g < nseg; ++g) {
    nS[g + 1] += nS[g];
    nE[g + 1] += nE[g];
    nW[g + 1] += nW[g];
  }
  desc.assign(4 * nS[nseg], 0);
  ids.assign(nE[nseg], 0);
  rows.assign(nW[nseg], 0);
  // pass 2: fill
#pragma omp parallel
  {
    std::vector<int64_t> key;
#pragma omp for schedule(dynamic, 16)
    for (int64_t g = 0; g < nseg; ++g) {
      segment_rows(quads, seg[g], seg[g + 1], rs, with_rows, key);
      int64_t S = nS[g], E = nE[g], Wr = nW[g];
      for (size_t a = 0; a < key.size();) {
        const int32_t m = kOgsMaxRowSize - (int32_t)(key[a] >> 32);
        size_t b = a;
        while (b < key.size() && (key[b] >> 32) == (key[a] >> 32)) ++b;
        const int64_t cap = 32LL * slab_rows_per_lane(m);
        for (size_t k0 = a; k0 < b; k0 += cap) {
          const int32_t n = (int32_t)std::min<int64_t>(cap, (int64_t)(b - k0));
          const int32_t nl = std::min(32, n);
          const int32_t Re = (n + nl - 1) / nl;
          const int32_t rem = n - (Re - 1) * nl;
          desc[4 * S + 0] = (int32_t)E;
          desc[4 * S + 1] = (int32_t)Wr;
          desc[4 * S + 2] = m;
          desc[4 * S + 3] = nl | (rem << 8) | (Re << 16);
          for (int32_t k = 0; k < n; ++k) {
            const int32_t j = k / nl, l = k % nl;
            const int32_t w = (j == Re - 1) ? rem : nl;
            const int32_t r = (int32_t)(uint32_t)key[k0 + k];
            for (int32_t t = 0; t < m; ++t)
              ids[E + (int64_t)j * m * nl + (int64_t)t * w + l] = ci[rs[r] + t];
            if (with_rows) rows[Wr + k] = perm ? perm[r] : r;
          }
          E += slab_span((int64_t)n * m);
          if (with_rows) Wr += n;
          ++S;
        }
        a = b;
      }
    }
  }
}

// 16-bit codes of the words of every slab g, words[first(g) .. first(g) + count(g))
// (compress_slabs, compress_slab_rows): a slab whose words have at most
// min(tableCap, 2^(16 - shift)) distinct high parts w >> shift gets a table of them
// (first-appearance order) and its words as (table index << shift | low bits); the
// others keep their 32-bit words.
template <typename Span>
static void code_slab_words(int64_t nslabs, Span span, const std::vector<int32_t>& words,
                            int shift, int32_t tableCap, std::vector<uint16_t>& codes,
                            std::vector<int32_t>& tables, std::vector<int32_t>& tdesc) {
  const int32_t maxTab = std::min<int32_t>(tableCap, 1 << (16 - shift));
  const int32_t mask = (1 << shift) - 1;
  codes.assign(words.size(), 0);
  tdesc.assign(2 * std::max<int64_t>(nslabs, 1), -1);
  std::vector<int64_t> ntab(nslabs + 1, 0);
  // pass 1: the distinct high parts of each slab (first-appearance order), codes
#pragma omp parallel
  {
    std::vector<int32_t> tab;
#pragma omp for schedule(dynamic, 64)
    for (int64_t g = 0; g < nslabs; ++g) {
      const std::pair<int64_t, int64_t> fc = span(g);
      tab.clear();
      bool ok = fc.second > 0;
      for (int64_t k = 0; k < fc.second && ok; ++k) {
        const int32_t word = words[fc.first + k], hi = word >> shift;
        int32_t t = 0;
        while (t < (int32_t)tab.size() && tab[t] != hi) ++t;
        if (t == (int32_t)tab.size()) {
          if ((int32_t)tab.size() == maxTab) ok = false;
          else tab.push_back(hi);
        }
        if (ok) codes[fc.first + k] = (uint16_t)((t << shift) | (word & mask));
      }
      ntab[g + 1] = ok ? (int32_t)tab.size() : 0;
      tdesc[2 * g + 1] = ok ? (int32_t)tab.size() : 0;
    }
  }
  for (int64_t g = 0; g < nslabs; ++g) ntab[g + 1] += ntab[g];
  if (ntab[nslabs] > INT32_MAX) {  // table offsets are 32-bit: leave every slab uncoded
    for (int64_t g = 0; g < nslabs; ++g) tdesc[2 * g + 1] = 0;
    tables.assign(1, 0);
    return;
  }
  tables.assign(std::max<int64_t>(ntab[nslabs], 1), 0);
  // pass 2: the tables (high part << shift), and each compressed slab's offset
#pragma omp parallel
  {
    std::vector<int32_t> tab;
#pragma omp for schedule(dynamic, 64)
    for (int64_t g = 0; g < nslabs; ++g) {
      if (tdesc[2 * g + 1] == 0) continue;
      const std::pair<int64_t, int64_t> fc = span(g);
      tab.clear();
      for (int64_t k = 0; k < fc.second; ++k) {
        const int32_t hi = words[fc.first + k] >> shift;
        if (std::find(tab.begin(), tab.end(), hi) == tab.end()) tab.push_back(hi);
      }
      for (size_t t = 0; t < tab.size(); ++t) tables[ntab[g] + t] = tab[t] << shift;
      tdesc[2 * g] = (int32_t)ntab[g];
    }
  }
}

// Rows of slab g: n = (Re - 1) * nl + rem.
static inline int64_t slab_nrows(const std::vector<int32_t>& desc, int64_t g) {
  const int32_t w = desc[4 * g + 3];
  return (int64_t)((w >> 16) - 1) * (w & 255) + ((w >> 8) & 255);
}

void compress_slabs(const std::vector<int32_t>& desc, const std::vector<int32_t>& ids, int shift,
                    std::vector<uint16_t>& codes, std::vector<int32_t>& tables,
                    std::vector<int32_t>& tdesc) {
  code_slab_words(
      (int64_t)desc.size() / 4,
      [&](int64_t g) {
        return std::make_pair((int64_t)desc[4 * g], slab_nrows(desc, g) * desc[4 * g + 2]);
      },
      ids, shift, kSlabCodeTable, codes, tables, tdesc);
}

void compress_slab_rows(const std::vector<int32_t>& desc, const std::vector<int32_t>& rows,
                        int shift, std::vector<uint16_t>& codes, std::vector<int32_t>& tables,
                        std::vector<int32_t>& tdesc) {
  code_slab_words(
      (int64_t)desc.size() / 4,
      [&](int64_t g) { return std::make_pair((int64_t)desc[4 * g + 1], slab_nrows(desc, g)); },
      rows, shift, kSlabRowTable, codes, tables, tdesc);
}

}  // namespace sp
