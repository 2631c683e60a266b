// Warp chunks of a gather-scatter operator and the order they are scheduled in.
//
// A chunk is a contiguous row range [r0, r1) holding at most kWarpChunkNnz
// non-zeros; one warp processes one chunk.  Any partition of the rows gives the
// same results (each row is summed by one lane in CSR order), so the partition and
// the chunk order are free to serve memory locality:
//   order 0 (natural): chunks follow the row order;
//   order 1 (bfs): rows are grouped by the 4 KiB page of local data holding their
//     first member, pages are visited breadth-first over the "row joins pages"
//     graph, and each page's rows are cut into chunks in that order.  Pages that
//     share rows are then processed close together in time, so the data one chunk
//     touches in a neighbouring page is usually still in L2 when that page's own
//     chunks run -- whatever the element numbering in memory.
#include <algorithm>
#include <vector>

#include "sp_ogs_plan.h"

namespace sp {

static constexpr int kPageShift = 9;  // 512 entries per page

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

bool build_chunks(int32_t nrows, const int32_t* rs, const int32_t* ci, int32_t ncols, int order,
                  std::vector<int32_t>& chunks) {
  chunks.clear();
  for (int32_t r = 0; r < nrows; ++r)
    if (rs[r + 1] - rs[r] > kWarpChunkNnz) return false;
  if (nrows == 0) return true;
  if (order == 0) {
    cut_run(0, nrows, rs, chunks);
    return true;
  }
  const int32_t npages = (std::max(ncols, 1) + (1 << kPageShift) - 1) >> kPageShift;
  // page of each row's first member; rows grouped by page (ascending row inside)
  std::vector<int32_t> pcount(npages + 1, 0);
  std::vector<int32_t> rowPage(nrows, -1);
  for (int32_t r = 0; r < nrows; ++r)
    if (rs[r + 1] > rs[r]) {
      rowPage[r] = ci[rs[r]] >> kPageShift;
      ++pcount[rowPage[r] + 1];
    }
  for (int32_t p = 0; p < npages; ++p) pcount[p + 1] += pcount[p];
  std::vector<int32_t> pageRows(pcount[npages]);
  {
    std::vector<int32_t> fill(pcount.begin(), pcount.end() - 1);
    for (int32_t r = 0; r < nrows; ++r)
      if (rowPage[r] >= 0) pageRows[fill[rowPage[r]]++] = r;
  }
  // undirected page graph: first page of a row -- page of each member
  std::vector<int32_t> stamp(npages, -1);
  std::vector<std::pair<int32_t, int32_t>> edges;
  for (int32_t p = 0; p < npages; ++p)
    for (int32_t k = pcount[p]; k < pcount[p + 1]; ++k) {
      const int32_t r = pageRows[k];
      for (int32_t i = rs[r]; i < rs[r + 1]; ++i) {
        const int32_t q = ci[i] >> kPageShift;
        if (q != p && stamp[q] != p) {
          stamp[q] = p;
          edges.emplace_back(p, q);
          edges.emplace_back(q, p);
        }
      }
    }
  std::sort(edges.begin(), edges.end());
  edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
  std::vector<int32_t> adjStart(npages + 1, 0);
  for (auto& e : edges) ++adjStart[e.first + 1];
  for (int32_t p = 0; p < npages; ++p) adjStart[p + 1] += adjStart[p];
  // breadth-first page order, restarting at the lowest unvisited page
  std::vector<uint8_t> seen(npages, 0);
  std::vector<int32_t> queue;
  queue.reserve(npages);
  for (int32_t start = 0; start < npages; ++start) {
    if (seen[start]) continue;
    seen[start] = 1;
    size_t head = queue.size();
    queue.push_back(start);
    while (head < queue.size()) {
      const int32_t p = queue[head++];
      for (int32_t k = adjStart[p]; k < adjStart[p + 1]; ++k) {
        const int32_t q = edges[k].second;
        if (!seen[q]) {
          seen[q] = 1;
          queue.push_back(q);
        }
      }
    }
  }
  // chunks: each page's rows as maximal contiguous runs, in page visit order
  for (int32_t p : queue) {
    int32_t k = pcount[p];
    while (k < pcount[p + 1]) {
      int32_t ra = pageRows[k], rb = ra + 1;
      ++k;
      while (k < pcount[p + 1] && pageRows[k] == rb) {
        ++rb;
        ++k;
      }
      cut_run(ra, rb, rs, chunks);
    }
  }
  // rows without members (possible in a caller-built CSR) still need a chunk
  for (int32_t r = 0; r < nrows; ++r)
    if (rowPage[r] < 0) {
      chunks.push_back(r);
      chunks.push_back(r + 1);
    }
  return true;
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
                  const int32_t* ci, const int32_t* ciE, std::vector<int32_t>& colS,
                  std::vector<uint8_t>& rowOf, std::vector<uint8_t>& e2s) {
  const int64_t nchunks = (int64_t)quads.size() / 4;
  const int32_t nnz = nrows > 0 ? rs[nrows] : 0;
  colS.assign(nnz, 0);
  rowOf.assign(nnz, 0);
  e2s.assign(nnz, 0);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t c = 0; c < nchunks; ++c) {
    const int32_t r0 = quads[4 * c], r1 = quads[4 * c + 1], g0 = quads[4 * c + 2];
    int64_t key[kWarpChunkNnz];  // column << 8 | row offset: sorts by column
    int32_t n = 0;
    for (int32_t r = r0; r < r1; ++r)
      for (int32_t i = rs[r]; i < rs[r + 1]; ++i) key[n++] = ((int64_t)ci[i] << 8) | (r - r0);
    std::sort(key, key + n);
    int32_t* cs = colS.data() + g0;
    for (int32_t j = 0; j < n; ++j) {
      cs[j] = (int32_t)(key[j] >> 8);
      rowOf[g0 + j] = (uint8_t)(key[j] & 0xFF);
    }
    // every column appears once in a chunk, so its sorted position is unique
    for (int32_t e = 0; e < n; ++e)
      e2s[g0 + e] = (uint8_t)(std::lower_bound(cs, cs + n, ciE[g0 + e]) - cs);
  }
}

}  // namespace sp
