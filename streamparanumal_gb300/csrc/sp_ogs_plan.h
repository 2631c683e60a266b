// Device-resident gather-scatter plan (the local ogsOperator_t of one rank).
#pragma once

#include <cstdint>
#include <vector>

#include "sp_internal.h"

namespace sp {

// Largest number of non-zeros one thread block stages (8 per lane of 256 lanes).
constexpr int kOgsThreads  = 256;
constexpr int kOgsPerLane  = 8;
constexpr int kOgsBlockNnz = kOgsThreads * kOgsPerLane;   // 2048
// The reference refuses groups larger than this (libs/ogs/ogsOperator.cpp:535).
constexpr int kOgsMaxRowSize = 512;
// Warp chunks: at most 256 non-zeros (8 per lane) and 256 rows, one warp each.
constexpr int kWarpChunkNnz = 256;
constexpr int kWarpsPerCta = 8;
// Resident CTAs per SM that the pipelined persistent gathers are compiled for (a
// register budget of 65536 / (256 * n) per lane) and launched with, and the one
// the column-order scatter is compiled for.  Build-time tuning values; GB300
// sweeps of the 64^3 p=7 box (3..6 and 5..8) put the optimum at 4 and 5.
#ifndef SP_OGS_PERSISTENT_CTAS
#define SP_OGS_PERSISTENT_CTAS 4
#endif
#ifndef SP_OGS_SCATTER_CTAS
#define SP_OGS_SCATTER_CTAS 5
#endif
constexpr int kOgsPersistentCtas = SP_OGS_PERSISTENT_CTAS;
// Resident CTAs per SM of the bulk-staged pipelined gathers (kernel 6): as many
// as kernel 2 (a fifth CTA leaves too few registers and spills).
constexpr int kOgsBulkCtas = 4;
constexpr int kOgsScatterCtas = SP_OGS_SCATTER_CTAS;

struct OgsOperatorDev {
  int32_t nrows = 0;       // rows covered by `blocks`
  int32_t nblocks = 0;
  int32_t* rowStarts = nullptr;  // nrows_padded + 1
  int32_t* colIds = nullptr;     // nnz
  int32_t* blocks = nullptr;     // nblocks + 1 row offsets
};

// Greedy partition of rows into blocks of at most kOgsBlockNnz non-zeros and at
// most kOgsBlockNnz rows.  Returns false when one row alone is too large.
bool partition_rows(int32_t nrows, const int32_t* rowStarts, std::vector<int32_t>& blocks);

// Cuts rows [0, nrows) into warp chunks, stored as (first row, end row) pairs in the
// order they are scheduled: 0 = row order, 1 = breadth-first over pages of
// 2^page_shift local entries (ball_shift > 0: a chain of breadth-first balls of
// 2^ball_shift entries).  Returns false when a row holds more than kWarpChunkNnz
// entries.  For order 1, `pages` (if given) receives the pages in visit order.
bool build_chunks(int32_t nrows, const int32_t* rowStarts, const int32_t* colIds, int32_t ncols,
                  int order, std::vector<int32_t>& chunks, int page_shift, int ball_shift,
                  std::vector<int32_t>* pages = nullptr);

// All rows in breadth-first page order: each page's rows (ascending) as the pages
// are visited, then rows without members.  seq[k] = the k-th row of the walk;
// `pages` (if given) receives the pages in visit order.
void bfs_row_sequence(int32_t nrows, const int32_t* rowStarts, const int32_t* colIds,
                      int32_t ncols, int page_shift, int ball_shift, std::vector<int32_t>& seq,
                      std::vector<int32_t>* pages = nullptr);

// Rows of every chunk regrouped by size.  `quads` holds the chunk descriptors
// (r0, r1, g0, g1).  Inside chunk [r0, r1) the rows are reordered by member count,
// largest first (ties in row order), and their members are laid out in that order
// over the chunk's own entry range [g0, g1), each row's members keeping their CSR
// order.  rowsG[r0 + k] = (offset of the k-th grouped row's first member from g0)
// | (its row - r0) << 16; colIdsG holds the regrouped column ids.  One warp then
// runs rows of equal size side by side, so its lanes finish their row loops
// together.
void build_grouped(const std::vector<int32_t>& quads, int32_t nrows, const int32_t* rowStarts,
                   const int32_t* colIds, std::vector<int32_t>& rowsG,
                   std::vector<int32_t>& colIdsG);

// Entries of every chunk in ascending column order, for kernels that touch local
// data in address order.  For chunk (r0, r1, g0, g1): colIdsS[g0 + j] is the j-th
// smallest column of the chunk and rowOfS[g0 + j] the offset from r0 of the row it
// belongs to (a scatter writes v[colIdsS[j]] = gv[r0 + rowOfS[j]] with neighbouring
// lanes on neighbouring addresses, and needs no row bounds).  The row walk of the
// gathers is CSR order (rowsG null, colIdsE = the CSR column ids) or grouped by
// size (rowsG and colIdsE from build_grouped); e2s[g0 + e] is the sorted position
// of entry e of that walk, so a gather can load values in column order and still
// combine each row in CSR order.
void build_sorted(const std::vector<int32_t>& quads, int32_t nrows, const int32_t* rowStarts,
                  const int32_t* rowsG, const int32_t* colIdsE, std::vector<int32_t>& colIdsS,
                  std::vector<uint8_t>& rowOfS, std::vector<uint8_t>& e2s);

// Lane-row slabs (kernel 7).  The rows of a walk (its chunks in visit order) are
// cut into segments of about 2^seg_shift entries; inside a segment the rows are
// regrouped by member count m (largest first, walk order kept within a size) and
// cut into slabs of at most 32 * R rows of one size, R = slab_rows_per_lane(m)
// rows per lane.  A slab of n rows uses nl = min(32, n) lanes and Re = ceil(n / nl)
// row steps; step j holds rows j*nl + l (lane l < nl, the last step only rem =
// n - (Re-1)*nl of them).  Member t of row (j, l) is ids[E + j*m*nl + t*w_j + l]
// with w_j = nl (rem for the last step): member-major, so the lanes' t-th loads
// are neighbouring words.  Each slab's ids start on a 16-byte boundary (up to 3
// unused words follow a slab whose entry count is not a multiple of 4), so a run
// of whole row steps can be copied in 16-byte pieces.  desc holds per slab (E, first
// row word, m, nl | rem << 8 | Re << 16); rows[first + j*nl + l] is the operator
// row of (j, l) (perm applied; only when `with_rows`, which also keeps the rows
// without members, as slabs of m = 0).  Each row keeps its members in CSR order.
constexpr int32_t kSlabLaneEntries = 16;
int32_t slab_rows_per_lane(int32_t m);

// 16-bit member ids for slabs (ogs.slab_code_shift = s): a slab whose ids have at
// most kSlabCodeTable distinct high parts (id >> s; and at most 2^(16-s)) stores
// each id as code = (index of its high part in the slab's table) << s | (id's low s
// bits), at the id's own position in `codes`; tables[tdesc[2g] + t] = high part t
// << s.  tdesc[2g + 1] = the table's length, 0 for a slab left uncompressed
// (tdesc[2g] = -1; it keeps its 32-bit ids).  On a box mesh of (p+1)^3 = 2^s local
// nodes per element a high part is an element, and a slab touches a few of them.
constexpr int32_t kSlabCodeTable = 128;
void compress_slabs(const std::vector<int32_t>& desc, const std::vector<int32_t>& ids, int shift,
                    std::vector<uint16_t>& codes, std::vector<int32_t>& tables,
                    std::vector<int32_t>& tdesc);
// The same codes for the row words of a gather walk's slabs (rows[first .. first +
// n) of slab g, n its rows), at their own positions in `codes`, with a table per
// slab of at most kSlabRowTable high parts (ogs.slab_row_codes).  The reference's
// first-appearance row order numbers the rows that first appear in one element
// consecutively, so a slab's rows, drawn from a few neighbouring elements, fall
// into a few runs (on hex boxes of p = 1..15 at most 32 for 93-100 % of the slabs).
constexpr int32_t kSlabRowTable = 32;
void compress_slab_rows(const std::vector<int32_t>& desc, const std::vector<int32_t>& rows,
                        int shift, std::vector<uint16_t>& codes, std::vector<int32_t>& tables,
                        std::vector<int32_t>& tdesc);
void build_slabs(const std::vector<int32_t>& quads, const int32_t* rs, const int32_t* ci,
                 const int32_t* perm, int seg_shift, bool with_rows, std::vector<int32_t>& desc,
                 std::vector<int32_t>& ids, std::vector<int32_t>& rows);

// Element slots of an nx*ny*nz box: slot[e] is where lexicographic element e is
// stored (identity for perm_seed 0, else a seeded Fisher-Yates shuffle).
std::vector<int32_t> box_slots(int64_t E, uint64_t perm_seed);

// Knuth MMIX linear congruential generator with the reference's constants and
// seeding (random.cpp:47-100): x_{n+1} = a*x_n + c (mod 2^64), state_0 = a*(~0 ^ seed) + c,
// draw = |(int)x| (low 32 bits as a signed int).
struct Lcg {
  static constexpr uint64_t A = 6364136223846793005ULL;
  static constexpr uint64_t C = 1ULL;
  uint64_t x;
  explicit Lcg(uint64_t seed) : x(A * (~0ULL ^ seed) + C) {}
  int32_t next_int() {
    const int32_t v = (int32_t)(uint32_t)x;
    x = A * x + C;
    // abs of INT_MIN stays INT_MIN in two's complement, as std::abs does in practice
    return (v < 0) ? (int32_t)(0u - (uint32_t)v) : v;
  }
};

}  // namespace sp

struct sp_ogs_plan {
  int32_t N = 0;
  int32_t NrowsT = 0, NrowsN = 0;
  int32_t nnzT = 0, nnzN = 0;
  int32_t maxRowSize = 0;
  bool n_is_t = false;            // N operator shares T's arrays

  std::vector<int32_t> rowStartsT, colIdsT;   // host copies, NrowsT+1 / nnzT
  std::vector<int32_t> rowStartsN, colIdsN;   // host copies, NrowsN+1 / nnzN

  // device arrays
  int32_t* d_rowStartsT = nullptr;   // NrowsT + 1
  int32_t* d_colIdsT = nullptr;      // nnzT
  int32_t* d_rowStartsNpad = nullptr;// NrowsT + 1 (rows >= NrowsN empty)
  int32_t* d_colIdsN = nullptr;      // nnzN
  int32_t* d_blocksT = nullptr;      // partition of T rows by T non-zeros
  int32_t* d_blocksN = nullptr;      // partition of N rows [0, NrowsN) by N non-zeros
  int32_t NrowBlocksT = 0, NrowBlocksN = 0;
  // warp chunks ((r0, r1) pairs) for the T and N operators; counts are 0 when a
  // row exceeds kWarpChunkNnz (the block kernels then serve every call)
  int32_t* d_chunksT = nullptr;
  int32_t* d_chunksN = nullptr;
  int32_t nchunksT = 0, nchunksN = 0;
  bool own_chunks_n = false;
  int32_t chunk_order = 0;
  // T rows regrouped by size inside each T chunk (build_grouped); null when the
  // plan keeps CSR order (knob ogs.rows = 0) or has no chunks
  int32_t* d_rowsGT = nullptr;       // NrowsT packed (start offset | row offset << 16)
  int32_t* d_colIdsGT = nullptr;     // nnzT
  int32_t row_order = 0;             // 1 when d_rowsGT / d_colIdsGT are in use
  // order 2: T rows renumbered in breadth-first page order (the walk the warp
  // kernels take), and each walk row's row of T; null otherwise (the walk is T)
  int32_t* d_walkRsT = nullptr;      // NrowsT + 1
  int32_t* d_walkCiT = nullptr;      // nnzT
  int32_t* d_permT = nullptr;        // NrowsT
  // T chunk entries in column order (build_sorted), for the column-order scatter
  int32_t* d_colIdsST = nullptr;     // nnzT
  uint8_t* d_rowOfST = nullptr;      // nnzT
  uint8_t* d_e2sT = nullptr;         // nnzT: sorted position of each row-order entry
  // the row of T holding each local column (-1: in no row), for the column-major
  // scatter; built with the warp chunks
  int32_t* d_rowOfColT = nullptr;    // N
  // pages of 2^pages_shift local columns in the main walk's visit order (chunk
  // orders 1 and 2), for the column-major scatter
  int32_t* d_pagesT = nullptr;
  int32_t npagesT = 0, pages_shift = 0;
  // optional second walk of T for the in-place gather+scatter (knob ogs.gs_order):
  // its own chunk order, page and ball sizes, rows grouped by size or the walk CSR
  int32_t* d_chunksGS = nullptr;
  int32_t nchunksGS = 0;
  int32_t gs_grouped = 0;
  int32_t* d_rsGS = nullptr;         // grouped rows, or the walk's row starts
  int32_t* d_ciGS = nullptr;         // grouped or walk column ids
  // per chunk (rows with more than one member, their entries) of the grouped main
  // walk and of the grouped gather+scatter walk (kernel 2's single-member path)
  int32_t* d_singT = nullptr;
  int32_t* d_singGS = nullptr;
  // lane-row slabs (kernel 7, knob ogs.slabs): of the main walk (descriptors, ids,
  // operator rows) and of the gather+scatter walk when the plan has one (no rows)
  int32_t* d_slabsT = nullptr;
  int32_t* d_slabIdsT = nullptr;
  int32_t* d_slabRowsT = nullptr;
  int32_t nslabsT = 0;
  int32_t* d_slabsGS = nullptr;
  int32_t* d_slabIdsGS = nullptr;
  int32_t nslabsGS = 0;
  // their 16-bit member codes (compress_slabs; null unless ogs.slab_code_shift > 0)
  uint16_t* d_slabCodesT = nullptr;
  int32_t* d_slabTabsT = nullptr;
  int32_t* d_slabTdT = nullptr;
  uint16_t* d_slabCodesGS = nullptr;
  int32_t* d_slabTabsGS = nullptr;
  int32_t* d_slabTdGS = nullptr;
  int32_t slab_code_shift = 0;
  int64_t slab_coded_entries = 0;   // entries in compressed slabs, both walks
  // the main walk's row words as 16-bit codes (compress_slab_rows; null unless
  // ogs.slab_row_codes with a code shift)
  uint16_t* d_slabRowCodesT = nullptr;
  int32_t* d_slabRowTabsT = nullptr;
  int32_t* d_slabRowTdT = nullptr;
  int64_t slab_coded_rows = 0;
  // count of bounded device waits that gave up (the bulk-staged gathers' waits)
  int32_t* d_waitErr = nullptr;
  bool own_n_csr = false;         // d_rowStartsNpad / d_colIdsN are separate allocations
  bool own_blocks_n = false;      // d_blocksN is a separate allocation

  int device = 0;
};
