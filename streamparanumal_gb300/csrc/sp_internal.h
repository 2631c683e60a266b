// Internal helpers shared by the CUDA translation units of libspgb300.so.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/sp_capi.h"

namespace sp {

// Records a formatted message as this host thread's last error and returns `s`.
sp_status fail(sp_status s, const char* fmt, ...);
// Clears the last error message.
void clear_error();
// Counts one kernel launch issued by the library on this host thread.
void count_launch(int64_t n = 1);

// Checks the launch that was just issued (configuration errors only: no sync).
inline sp_status check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(SP_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  count_launch();
  return SP_SUCCESS;
}

inline cudaStream_t as_cuda(sp_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

#define SP_CUDA_TRY(expr)                                                              \
  do {                                                                                 \
    cudaError_t _e = (expr);                                                           \
    if (_e != cudaSuccess)                                                             \
      return ::sp::fail(SP_ERR_CUDA, "%s failed: %s", #expr, cudaGetErrorString(_e));  \
  } while (0)

// Number of SMs of the current device (cached per device).
int sm_count();

// ---------------------------------------------------------------- tuning knobs
// Runtime-selectable launch parameters (the autotuner's surface, sp_tune_set/get).
enum TuneKey : int {
  kTuneReducePrefetch = 0,  // order-exact reductions: L2 prefetch distance in chunks (-1 = per kernel)
  kTuneOgsBlockNnz,         // ogs plan: non-zeros per row block (256 .. 2048), read at plan creation
  kTuneOgsKernel,           // ogs gather+scatter: 0 block, 1 warp-chunk, 2 pipelined, 3 async-staged, ..., 7 lane-row slabs (k == 1)
  kTuneOgsOrder,            // ogs plan: warp-chunk order, 0 = rows, 1 = breadth-first pages
  kTuneReduceRolling,       // order-exact reductions: 1 = rolling load pipeline, 0 = grouped
  kTuneOgsKernelGather,     // ogs gather: kernel variant as kTuneOgsKernel
  kTuneOgsKernelScatter,    // ogs scatter: kernel variant as kTuneOgsKernel
  kTuneOgsRows,             // ogs plan: rows inside a warp chunk, 0 = CSR order, 1 = grouped by size
  kTuneOgsPageShift,        // ogs plan: log2 of the page size of the breadth-first chunk order
  kTuneOgsBallShift,        // ogs plan: 0 breadth-first pages, else balls of 2^n entries
  kTuneOgsGsOrder,          // ogs plan: -1 gather+scatter on the main walk, else its own walk's order
  kTuneOgsGsPageShift,      // ogs plan: page size of the gather+scatter walk
  kTuneOgsGsBallShift,      // ogs plan: ball size of the gather+scatter walk
  kTuneOgsScatterPages,     // ogs column-major scatter: 1 = pages in the main walk's order
  kTuneNormExact,           // BS3 at the drivers' bs3_1 call sites: 0 integer-pipe norm, 1 order-exact
  kTuneNormCtas,            // integer-pipe norm: resident CTAs per SM (4 or 6)
  kTuneNormRoll,            // integer-pipe norm: 1 = rolling load pipeline
  kTuneOgsSingles,          // ogs kernel 2: 1 = single-member rows skip staging and combine
  kTuneRdotrExact,          // BS5 at the drivers' bs5_1 call sites: 0 integer-pipe r.r, 1 order-exact
  kTuneOgsSlabs,            // ogs plan: 1 = build the lane-row slab layouts (kernel 7)
  kTuneOgsSlabSegShift,     // ogs plan: log2 of the entries regrouped together into slabs
  kTuneOgsSlabLane,         // kernel 7: members in flight per lane (0 per type, 8 or 16)
  kTuneOgsSlabCtas,         // kernel 7: resident CTAs per SM (0 = 2, 1..4)
  kTuneOgsSlabLoad,         // kernel 7: value loads 0 plain, 1 L2 only, 2 evict-first, 3 read-only path
  kTuneOgsSlabDefer,        // kernel 7 gather+scatter: 1 = a pass's stores after the next pass's loads
  kTuneOgsSlabCodeShift,    // ogs plan: 0 = 32-bit slab ids, 6..12 = 16-bit codes with that many low bits
  kTuneOgsKernel32,         // ogs gather+scatter of 4-byte values: kernel variant, -1 = as ogs.kernel
  kTuneOgsKernelGather32,   // ogs gather of 4-byte values: kernel variant, -1 = as ogs.kernel.gather
  kTuneOgsSlabRowCodes,     // ogs plan: 1 = with member codes, the gather slabs' row words coded too (default 0)
  kTuneCount
};
int64_t tune(TuneKey k);

// ---------------------------------------------------------------- scratch layout
// Layout of the caller-provided scratch of the single-launch reductions:
//   [0, 8)                          : unsigned int ticket counter (+4 bytes pad)
//   [256, 256 + 32*kMaxRedBlocks)   : per-block partials, 32 bytes per block (two
//                                     doubles, or the integer-pipe accumulator)
constexpr int    kMaxRedBlocks   = 2048;
constexpr size_t kRedPartialOff  = 256;
constexpr size_t kRedPartialBytes = 32;
constexpr size_t kRedScratchSize = kRedPartialOff + kRedPartialBytes * (size_t)kMaxRedBlocks;

}  // namespace sp
