/*
 * sp_capi.h -- C ABI of the GB300 (sm_103a) streaming hot path of streamParanumal.
 *
 * This is the boundary that replaces the OCCA device behind the reference's
 * platform_t / kernel_t / deviceMemory<T> / ogs::ogs_t objects.  Every entry point
 * takes plain pointers and sizes, runs on an explicit CUDA stream, and returns an
 * sp_status instead of throwing (the reference aborts through LIBP_ABORT,
 * include/utils.hpp:69; the C++ mirror in streamparanumal_gb300/host turns a
 * non-success status back into that exception).
 *
 * Conventions
 *  - Device pointers are plain CUDA device addresses.  Host pointers are named
 *    h_* and are only read during the call.
 *  - All launches are asynchronous on `stream` (NULL = legacy default stream).
 *    No entry point synchronises the device except the *_create/setup calls,
 *    which copy plan data to the device.
 *  - Vector lengths are int64_t; ogs indices are int32_t (the reference's dlong,
 *    include/types.h:60) and ogs ids are int64_t (hlong, include/types.h:52).
 *  - After a failing call, sp_last_error_string() describes the failure
 *    (per host thread).
 */
#ifndef SP_CAPI_H
#define SP_CAPI_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* sp_stream_t; /* identical to cudaStream_t */

typedef int32_t sp_status;
#define SP_SUCCESS            0
#define SP_ERR_INVALID_ARG    1  /* null pointer, negative size, bad enum          */
#define SP_ERR_CUDA           2  /* a CUDA runtime call or launch failed            */
#define SP_ERR_ALLOC          3  /* cudaMalloc / host allocation failed             */
#define SP_ERR_UNSUPPORTED    4  /* a type/op/transpose combination not provided    */
#define SP_ERR_SIZE           5  /* size exceeds an int32 index or a plan limit     */
#define SP_ERR_CSR            6  /* malformed CSR / ids handed to a plan builder    */
#define SP_ERR_TIMEOUT        7  /* a bounded device-side wait gave up              */
#define SP_ERR_DEVICE_CHECK   8  /* a device-side bounds check recorded a bad index */

/* ogs enums: same values as the reference's ogs::Type / Op / Transpose / Kind
 * (include/ogs.hpp:179-200). */
typedef enum { SP_FLOAT = 0, SP_DOUBLE = 1, SP_INT32 = 2, SP_INT64 = 3 } sp_type;
typedef enum { SP_OP_ADD = 0, SP_OP_MUL = 1, SP_OP_MAX = 2, SP_OP_MIN = 3 } sp_op;
typedef enum { SP_SYM = 0, SP_NOTRANS = 1, SP_TRANS = 2 } sp_transpose;
typedef enum { SP_KIND_UNSIGNED = 0, SP_KIND_SIGNED = 1, SP_KIND_HALO = 2 } sp_kind;

/* ---------------------------------------------------------------- library */
const char* sp_last_error_string(void);
const char* sp_status_string(sp_status s);
int32_t     sp_version(void);                 /* 10000*major + 100*minor + patch */
/* Number of kernel launches issued by this library on the calling host thread
 * since the last reset (used by harnesses to count launches in a timed region). */
int64_t     sp_launch_count(void);
void        sp_launch_count_reset(void);
/* Tuning knobs selecting among compiled kernel variants (process-wide; the
 * autotuner's surface).  Every variant computes the same bits, except under
 * "reduce.norm_exact" (a different, more accurate summation of BS3).  Keys:
 *  "reduce.prefetch_chunks" (-1..64, default -1 = per-kernel defaults): L2
 *    bulk-prefetch distance of the order-exact reductions;
 *  "reduce.rolling" (1 rolling load pipeline, 0 grouped loads; default 1) for the
 *    order-exact reductions;
 *  "ogs.block_nnz" (256..2048, default 2048): non-zeros per row block of plans
 *    created afterwards;
 *  "ogs.order" (0 row order, 1 breadth-first over pages of local data, 2 rows
 *    renumbered in that breadth-first order so that chunks are full; default 1),
 *    "ogs.page_shift" (3..16, default 9: pages of 2^9 entries) and "ogs.rows" (0
 *    CSR order, 1 rows grouped by size inside a chunk; default 1) for the warp
 *    chunks of plans created afterwards; "ogs.ball_shift" (0 = pages visited
 *    breadth-first over the whole mesh, 1..26 = as a chain of breadth-first balls
 *    of 2^n entries; default 0);
 *  "ogs.gs_order" (-1 = the gather+scatter uses the main walk; 0..2 = plans
 *    created afterwards also hold a second walk of T in that order, used by the
 *    in-place gather+scatter; default -1), "ogs.gs_page_shift" (3..16, default 8)
 *    and "ogs.gs_ball_shift" (0..26, default 18) for that walk;
 *  "ogs.kernel" / "ogs.kernel.gather" / "ogs.kernel.scatter" (gather+scatter /
 *    gather / scatter): 0 block kernels, 1 warp-chunk kernels, 2 pipelined
 *    persistent warp-chunk kernels, 3 asynchronously staged gathers (cp.async) or
 *    the column-order scatter, 4 column-order pipelined gathers or the persistent
 *    column-order scatter with L2 prefetch, 5 pipelined gathers with L2 prefetch or
 *    the column-major scatter (one thread per local column), 6 (gathers only) the
 *    pipelined gathers with each chunk's column ids staged in shared memory by TMA
 *    bulk copy one chunk ahead, 7 (gather and gather+scatter) lane-row slabs: each
 *    lane combines whole rows in registers, rows of one size side by side, from the
 *    plan's slab layout (no shared memory); defaults 2, 2, 5; "ogs.kernel.f32" and
 *    "ogs.kernel.gather.f32" (-1..7, default -1 = as the two above) choose the
 *    gather+scatter and gather kernels of 4-byte values separately;
 *  "ogs.slabs" (1 = plans created afterwards also hold the slab layouts kernel 7
 *    runs on, about 4 bytes per entry and per row of each walk; default 0: kernel
 *    7 then runs as kernel 2), "ogs.slab_seg_shift" (8..22, default 17: rows are
 *    regrouped by size inside runs of 2^n entries of the walk), "ogs.slab_code_shift"
 *    (0..12, default 0: with s > 0 a slab whose ids have at most 128 distinct high
 *    parts id >> s stores them as 16-bit codes (table index << s | low s bits),
 *    which kernel 7 decodes through the slab's table; s = log2 of the nodes per
 *    element, e.g. 9 at p = 7, makes a high part an element), "ogs.slab_row_codes"
 *    (0..1, default 0: with s > 0 the gather's slabs also hold the output row of
 *    each of their rows as such a code, decoded through a second table per slab
 *    of at most 32 runs by kernel 7's default Add gather; measured on GB300 +8 %
 *    FP64 at p = 5 on permuted boxes, -4 % at p = 7 and -12 % for FP32, hence off);
 *  "ogs.slab_lane" (0..16, default 0: members in flight per lane and pass of
 *    kernel 7 -- 0 = 8, and 16 for the gather+scatter of 4-byte values, 1..8 = 8,
 *    9..16 = 16), "ogs.slab_ctas" (0..4, default 0: resident CTAs of 256
 *    lanes per SM kernel 7 is compiled and launched for; 0 = 3 for 4-byte values
 *    at 8 members per lane, else 2) and
 *    "ogs.slab_load" (0..3, default 0: kernel 7's value loads -- 0 plain, 1 L2
 *    only, 2 evict-first, 3 the read-only path for gathers, plain for the in-place
 *    gather+scatter; with the default CTAs) and "ogs.slab_defer" (1 = kernel 7's
 *    in-place gather+scatter stores a pass's results after the next pass's loads;
 *    default 1), all for the Add op (other ops run the defaults);
 *  "ogs.singles" (0..2, default 2; kernel 2 on rows grouped by size: 1 = the
 *    in-place gather+scatter lets the rows of a single member skip the
 *    shared-memory staging and the combine loop -- the lane that gathered such a
 *    value applies the op's first step and stores it back only when that changed
 *    its bits (-0 under Add, -Inf or NaN under Max/Min), so memory ends the same
 *    and unchanged values are not rewritten; 2 = as 1, and the gathers write
 *    single-member rows from the gathering lane too);
 *  "ogs.scatter_pages" (1 = the column-major scatter takes the pages of local
 *    columns in the main walk's order when the plan has one (chunk orders 1 and 2)
 *    and a page holds at least 1 KiB of values, 0 = in memory order; default 1);
 *  "reduce.norm_exact" (0 = the C++ platform's bs3_1 binding runs the integer-pipe
 *    norm sp_bs3_1_fast_f64, 1 = the order-exact sp_bs3_1_f64; default 0);
 *  "reduce.rdotr_exact" (0 = the C++ platform's bs5_1 binding runs
 *    sp_bs5_1_fast_f64, 1 = the order-exact sp_bs5_1_f64; default 0);
 *  "reduce.norm_ctas" (4 or 6, default 4): resident CTAs of 256 lanes per SM, and
 *    CTAs per SM of the persistent grid, of the integer-pipe norm (values 5 run 4);
 *  "reduce.norm_roll" (1 = the integer-pipe norm keeps the next loads of each lane
 *    in flight while it adds the current ones; default 1).
 * Unknown keys or out-of-range values return SP_ERR_INVALID_ARG. */
sp_status   sp_tune_set(const char* key, int64_t value);
sp_status   sp_tune_get(const char* key, int64_t* value);

/* ---------------------------------------------------------------- BS0
 * Empty 1x1 launch.  Replaces the `bs0` kernel (BS/BS0/okl/bs0.okl:27-39) launched
 * by bs0_t::Run (BS/BS0/src/bs0Run.cpp:72). Writes b[0]=0 only if n==0. */
sp_status sp_bs0(int32_t n, const double* a, double* b, sp_stream_t stream);

/* BS0 graph form: capture `nlaunches` empty kernels into one CUDA graph once,
 * then replay it with a single launch (collapses the per-launch host cost). */
typedef struct sp_graph sp_graph;
sp_status sp_bs0_graph_create(int32_t nlaunches, int32_t n, const double* a, double* b,
                              sp_stream_t stream, sp_graph** out);
/* Capture everything this host thread launches on `stream` (a created stream, not
 * the legacy default one) between sp_graph_begin and sp_graph_end into one graph;
 * replay it with sp_graph_launch.  Plans and buffers must exist before capture. */
sp_status sp_graph_begin(sp_stream_t stream);
sp_status sp_graph_end(sp_stream_t stream, sp_graph** out);
sp_status sp_graph_launch(const sp_graph* g, sp_stream_t stream);
sp_status sp_graph_destroy(sp_graph* g);

/* ---------------------------------------------------------------- BS1 copy
 * b[n] = a[n].  Replaces `bs1` (BS/BS1/okl/bs1.okl:27-34), called at
 * BS/BS1/src/bs1Run.cpp:76 as kernel(N, o_a, o_b).  Bit-exact. */
sp_status sp_bs1_copy_f64(int64_t n, const double* a, double* b, sp_stream_t stream);
sp_status sp_bs1_copy_f32(int64_t n, const float* a, float* b, sp_stream_t stream);

/* ---------------------------------------------------------------- BS2 axpy
 * y[n] = alpha*x[n] + beta*y[n].  Replaces `bs2` (BS/BS2/okl/bs2.okl:27-36),
 * called at BS/BS2/src/bs2Run.cpp:79 as kernel(N, alpha, o_x, beta, o_y).
 * FP64 rounding follows the reference's CUDA mode (--fmad=true,
 * libs/core/platformProperties.cpp:76): y = fma(alpha, x, beta*y). */
sp_status sp_bs2_axpy_f64(int64_t n, double alpha, const double* x, double beta, double* y,
                          sp_stream_t stream);
sp_status sp_bs2_axpy_f32(int64_t n, float alpha, const float* x, float beta, float* y,
                          sp_stream_t stream);

/* ---------------------------------------------------------------- BS3/BS4/BS5
 * Order-exact two-stage reductions: the same partition and summation tree as the
 * reference's kernels, so results are bit-identical to its CUDA mode.
 *   stage 1: nblocks logical blocks of `block_size` (256 or 1024) lanes; lane t of
 *            block b accumulates ids t + b*bs + j*bs*nblocks in order, then a
 *            halving tree writes partial[b].
 *   stage 2: one block sums partial[0..nblocks) with the same tree into out[0].
 * BS3  bs3_1/bs3_2 (BS/BS3/okl/bs3.okl:27-102; call sites bs3Run.cpp:83-84):
 *        partial = sum a*a                      (no sqrt)
 * BS4  bs4_1/bs4_2 (BS/BS4/okl/bs4.okl:27-103; bs4Run.cpp:83-84):  sum a*b
 * BS5  bs5_1/bs5_2 (BS/BS5/okl/bs5.okl:27-106; bs5Run.cpp:87-88):
 *        r = r + alpha*Ap (stored), partial = sum r*r
 * nblocks must be in [1, block_size]; block_size in {256, 512, 1024}. */
sp_status sp_bs3_1_f64(int32_t block_size, int32_t nblocks, int64_t n, const double* a,
                       double* partial, sp_stream_t stream);
sp_status sp_bs4_1_f64(int32_t block_size, int32_t nblocks, int64_t n, const double* a,
                       const double* b, double* partial, sp_stream_t stream);
sp_status sp_bs5_1_f64(int32_t block_size, int32_t nblocks, int64_t n, const double* Ap,
                       double alpha, double* r, double* partial, sp_stream_t stream);
/* Stage 2, shared by bs3_2 / bs4_2 / bs5_2 (identical kernels in the reference). */
sp_status sp_reduce_finish_f64(int32_t block_size, int32_t nblocks, const double* partial,
                               double* out, sp_stream_t stream);

/* ---------------------------------------------------------------- allocation-free dot
 * No counterpart in the reference.  The BS4 dot (bs4_1 then bs4_2, bit-identical to
 * sp_bs4_1_f64 + sp_reduce_finish_f64) for callers that cannot allocate device
 * memory -- their device memory belongs to another allocator or a fixed pool, or
 * they cannot afford cudaMalloc's device-wide synchronisation -- and therefore
 * cannot supply the partial-sum buffer.  The partials live in a static 1024-double
 * array inside the library (8 KiB held on every GPU that loads it, until exit):
 *  - nblocks must not exceed 1024 (larger values fail with SP_ERR_SIZE);
 *  - the first call on a device looks up the array's device address (set-up);
 *    make that first call before any stream capture.  The address is kept per
 *    device ordinal for the life of the process: after cudaDeviceReset() (which
 *    destroys the context the address belongs to) do not call this entry point
 *    again in that process;
 *  - every call shares the one array, so calls that overlap on the GPU (other
 *    streams, other host threads) race; serialise them on one stream;
 *  - nothing in the array has to start at zero: each call writes the partials it
 *    reads.  Allocates nothing. */
sp_status sp_bs4_dot_f64_noalloc(int32_t block_size, int32_t nblocks, int64_t n, const double* a,
                                 const double* b, double* out, sp_stream_t stream);

/* ---------------------------------------------------------------- fast reductions
 * Single-launch reductions over a fixed grid (deterministic for a given n, but
 * not the reference's summation order).  `scratch` must hold
 * sp_reduce_scratch_bytes() bytes and be zero-filled before its first use; every
 * call leaves it zero-filled again.  Calls sharing one scratch must not overlap
 * on the device.  Results go to the device scalar out[0] (FP64).
 * FP32-storage forms accumulate in FP32 with compensated (TwoSum) per-lane
 * partials and finalise across blocks in FP64. */
size_t    sp_reduce_scratch_bytes(void);
/* FP64 sum of squares with the per-element work on the integer pipe: each lane
 * accumulates the squared significands in 128-bit fixed point relative to its
 * largest exponent (elements more than 15 binades below it, subnormals, Inf and
 * NaN go to an FP64 fma side sum), lanes and blocks are combined in double-double.
 * The result is within a few ulps of the exactly rounded sum for every input
 * (Inf/NaN/overflow as FP64 gives them), hence within 1e-14 relative of the
 * reference's order-exact bs3 (BS/BS3/okl/bs3.okl:36-41). */
sp_status sp_norm2_f64(int64_t n, const double* a, double* out, void* scratch, sp_stream_t stream);
/* Stage 1 of BS3 in that form, for the call sites of bs3_1 (BS/BS3/src/bs3Run.cpp:83):
 * partial[0] = sum a*a as sp_norm2_f64 computes it and partial[1 .. nblocks) = 0,
 * so that the unchanged stage 2 (bs3_2 = sp_reduce_finish_f64 over nblocks
 * partials) returns partial[0].  block_size and nblocks as for sp_bs3_1_f64;
 * scratch as above.  This is the BS3 default of the drivers and the benchmark; the
 * order-exact sp_bs3_1_f64 stays available (knob "reduce.norm_exact"). */
sp_status sp_bs3_1_fast_f64(int32_t block_size, int32_t nblocks, int64_t n, const double* a,
                            double* partial, void* scratch, sp_stream_t stream);
/* Stage 1 of BS5 in the same form, for the call sites of bs5_1 (BS/BS5/src/bs5Run.cpp:87):
 * r = fma(alpha, Ap, r) as sp_bs5_1_f64 stores it (the same bits), partial[0] = sum r*r
 * over the stored r on the integer pipe (as sp_norm2_f64: within a few ulps of the
 * exactly rounded sum, hence within 1e-14 relative of the reference's order-exact
 * bs5_1/bs5_2, BS/BS5/okl/bs5.okl:27-106) and partial[1 .. nblocks) = 0, so that the
 * unchanged stage 2 returns partial[0].  One FP64 fma per entry instead of two: the
 * order-exact form is bound by GB300's FP64 pipe and HBM together.  The drivers'
 * default; the order-exact sp_bs5_1_f64 stays available (knob "reduce.rdotr_exact").
 * block_size and nblocks as for sp_bs5_1_f64; scratch as above. */
sp_status sp_bs5_1_fast_f64(int32_t block_size, int32_t nblocks, int64_t n, const double* Ap,
                            double alpha, double* r, double* partial, void* scratch,
                            sp_stream_t stream);
sp_status sp_dot_f64(int64_t n, const double* a, const double* b, double* out, void* scratch,
                     sp_stream_t stream);
sp_status sp_norm2_f32(int64_t n, const float* a, double* out, void* scratch, sp_stream_t stream);
sp_status sp_dot_f32(int64_t n, const float* a, const float* b, double* out, void* scratch,
                     sp_stream_t stream);

/* ---------------------------------------------------------------- CG update
 * Full CG update (x, r and r.r in one pass; the reference's BS5 only does the r update):
 *   x += alpha*p;  r -= alpha*Ap;  rdotr[0] = sum r*r   (FP64 result)
 * x = fma(alpha, p, x), r = fma(-alpha, Ap, r), accumulation fma(r, r, acc).
 * Scratch rules as for the fast reductions. */
sp_status sp_cg_update_f64(int64_t n, double alpha, const double* p, const double* Ap,
                           double* x, double* r, double* rdotr, void* scratch,
                           sp_stream_t stream);
sp_status sp_cg_update_f32(int64_t n, double alpha, const float* p, const float* Ap,
                           float* x, float* r, double* rdotr, void* scratch,
                           sp_stream_t stream);
/* The reference's BS5 update (BS/BS5/okl/bs5.okl:27-106) in one launch over the
 * fixed grid of the fast reductions: r = fma(alpha, Ap, r) (FP32: fmaf with alpha
 * rounded to FP32), rdotr[0] = sum r*r (FP64: deterministic, not the reference's
 * order; FP32: compensated FP32 lanes, FP64 finish).  Scratch rules as above. */
sp_status sp_cg_update_ref_f64(int64_t n, double alpha, const double* Ap, double* r,
                               double* rdotr, void* scratch, sp_stream_t stream);
sp_status sp_cg_update_ref_f32(int64_t n, double alpha, const float* Ap, float* r,
                               double* rdotr, void* scratch, sp_stream_t stream);

/* ---------------------------------------------------------------- ogs
 * A gather-scatter plan is the device form of the reference's local
 * ogsOperator_t (include/ogs/ogsOperator.hpp:44-138): a T operator (all members
 * of each group) and an N operator (positive members only) in CSR, plus a row
 * partition into blocks of at most sp_ogs_block_nnz() non-zeros.
 * Rows/columns follow ogsBase_t::Setup (libs/ogs/ogsSetup.cpp:87-290): rows are
 * groups in order of first appearance (positive groups first), columns ascending
 * local index inside each row.  Sums run in that column order from the op's
 * identity, so FP64/FP32 results are bit-identical to the reference. */
typedef struct sp_ogs_plan sp_ogs_plan;

typedef struct {
  int32_t N;          /* local vector length the plan acts on                  */
  int32_t NrowsT;     /* rows of the T operator (= Ngather on one rank)         */
  int32_t NrowsN;     /* rows with a positive member                           */
  int32_t nnzT;       /* entries in the T operator                             */
  int32_t nnzN;       /* entries in the N operator                             */
  int32_t NrowBlocksT;
  int32_t NrowBlocksN;
  int32_t maxRowSize; /* largest group                                          */
  int64_t NgatherGlobal;
  int32_t NchunksT;   /* warp chunks of the T / N operators (0: block kernels only) */
  int32_t NchunksN;
  int32_t chunkOrder; /* 0 row order, 1 breadth-first pages, 2 renumbered walk     */
  int32_t rowOrder;   /* T rows inside a chunk: 0 CSR order, 1 grouped by size      */
  int32_t NchunksGS;  /* chunks of the gather+scatter's own walk (0: none)         */
  int32_t gsRowOrder; /* its rows: 0 CSR order, 1 grouped by size                  */
  int32_t NpagesT;    /* pages of local columns in the main walk's order (0: none)  */
  int32_t pageShift;  /* log2 of their size in columns                              */
  int32_t waitErrors; /* bounded device waits of this plan's kernels that gave up
                         (kernel 6's staging waits; 0 in every correct run; reading it
                         synchronises the device)                                  */
  int32_t NslabsT;    /* lane-row slabs of the main walk (kernel 7; 0: not built)   */
  int32_t NslabsGS;   /* lane-row slabs of the gather+scatter walk (0: none)         */
  int32_t slabCodeShift;    /* low bits of the slabs' 16-bit member codes (0: none)  */
  int64_t slabCodedEntries; /* entries of both walks' slabs held as 16-bit codes      */
  int64_t slabCodedRows;    /* gather rows whose row word is held as a 16-bit code     */
} sp_ogs_info;

/* Build from global ids (ogs_t::Setup, include/ogs.hpp:221-228 at one rank):
 * h_ids[N] (0 = ignored, negative = flagged).  With unique != 0 exactly one member
 * of every group is made positive and the signs are written back into h_ids
 * (as the reference does).  Host-side setup plus device upload on `stream`. */
sp_status sp_ogs_setup(int32_t N, int64_t* h_ids, sp_kind kind, int32_t unique,
                       sp_stream_t stream, sp_ogs_plan** out);
/* The same setup with the ids in device memory (d_ids[N], signs written back there
 * with unique): grouping, owner draws, row numbering and CSR built on the GPU
 * (same plan as sp_ogs_setup), for meshes whose ids are generated on the device.
 * Allocates scratch of about 60 bytes per id; synchronises `stream`. */
sp_status sp_ogs_setup_device(int32_t N, int64_t* d_ids, sp_kind kind, int32_t unique,
                              sp_stream_t stream, sp_ogs_plan** out);
/* Host half of sp_ogs_setup: fills the T and N CSR without touching the device.
 * rowStarts* need N+1 entries and colIds* N entries. */
sp_status sp_ogs_setup_csr(int32_t N, int64_t* h_ids, sp_kind kind, int32_t unique,
                           int32_t* NrowsT, int32_t* h_rowStartsT, int32_t* h_colIdsT,
                           int32_t* NrowsN, int32_t* h_rowStartsN, int32_t* h_colIdsN);
/* Build from an explicit CSR (T operator) and optional N operator.  Passing NULL
 * h_rowStartsN/h_colIdsN makes the N operator share T's CSR over T's first NrowsN
 * rows (NrowsN < 0 or > NrowsT: all rows), as for an Unsigned handle. */
sp_status sp_ogs_plan_create(int32_t N, int32_t NrowsT, const int32_t* h_rowStartsT,
                             const int32_t* h_colIdsT, int32_t NrowsN,
                             const int32_t* h_rowStartsN, const int32_t* h_colIdsN,
                             sp_stream_t stream, sp_ogs_plan** out);
sp_status sp_ogs_plan_destroy(sp_ogs_plan* plan);
sp_status sp_ogs_plan_info(const sp_ogs_plan* plan, sp_ogs_info* info);
/* Copy the host CSR of one operator (trans = SP_TRANS -> T, SP_NOTRANS -> N) into
 * caller arrays sized NrowsX+1 and nnzX (either pointer may be NULL). */
sp_status sp_ogs_plan_csr(const sp_ogs_plan* plan, sp_transpose which, int32_t* h_rowStarts,
                          int32_t* h_colIds);
int32_t   sp_ogs_block_nnz(void);

/* ogs_t::Gather   (include/ogs.hpp:289-293; libs/ogs/ogs.cpp:205-301;
 *                  kernel libs/ogs/okl/ogsKernels.okl:86-122)
 *   gv[row*k + f] = op over members c of row (CSR order) of v[col(c)*k + f]
 *   trans == SP_NOTRANS uses the N operator, otherwise T.
 * ogs_t::Scatter  (include/ogs.hpp:327-330; ogs.cpp:394-492; ogsKernels.okl:127-164)
 *   v[col(c)*k + f] = gv[row*k + f]; trans == SP_TRANS uses N, otherwise T.
 * ogs_t::GatherScatter (include/ogs.hpp:251-254; ogs.cpp:39-125; ogsKernels.okl:32-81)
 *   Sym: gather T / scatter T; NoTrans: gather N / scatter T; Trans: gather T /
 *   scatter N.  The op is honoured for every transpose (the reference's device
 *   path always uses Add, libs/ogs/ogsOperator.cpp:448). */
sp_status sp_ogs_gather(const sp_ogs_plan* plan, sp_type type, sp_op op, sp_transpose trans,
                        int32_t k, void* gv, const void* v, sp_stream_t stream);
sp_status sp_ogs_scatter(const sp_ogs_plan* plan, sp_type type, sp_transpose trans, int32_t k,
                         void* v, const void* gv, sp_stream_t stream);
sp_status sp_ogs_gather_scatter(const sp_ogs_plan* plan, sp_type type, sp_op op,
                                sp_transpose trans, int32_t k, void* v, sp_stream_t stream);

/* ---------------------------------------------------------------- multi-rank ogs
 * ogs_t::Setup over a communicator of several ranks (libs/ogs/ogsSetup.cpp:87-290:
 * FindSharedGroups :292-469, ConstructSharedNodes :617-813) with the Pairwise
 * exchange (libs/ogs/ogsPairwise.cpp:176-387).  Each rank holds its own local
 * nodes.  Groups whose members all sit on this rank form the local operator, groups
 * shared with other ranks the halo operator; a pairwise exchange of gathered halo
 * rows joins the halo groups across ranks.  The library has no transport of its
 * own: setup talks through the caller's sp_comm callbacks, and the data exchange is
 * made by the caller between sp_ogs_mr_exchange_start and sp_ogs_mr_exchange_finish,
 * following sp_ogs_mr_schedule (one message per peer and direction, as the
 * Isend/Irecv pairs of ogsPairwise_t::DeviceFinish, ogsPairwise.cpp:125-156).
 *
 * Callbacks return 0 on success (anything else fails the setup with SP_ERR_COMM).
 *   alltoallv: this rank sends sendcounts[r] elements of elem_bytes bytes, from
 *     element sdispls[r] of `send`, to rank r and receives recvcounts[r] elements
 *     from rank r at element rdispls[r] of `recv` (MPI_Alltoallv);
 *   allreduce_i64: *value <- op over all ranks (op 0 sum, 1 min, 2 max). */
#define SP_ERR_COMM           9  /* an sp_comm callback reported a failure          */
typedef struct {
  int32_t rank;
  int32_t size;
  void* ctx;
  int32_t (*alltoallv)(void* ctx, const void* send, const int64_t* sendcounts,
                       const int64_t* sdispls, void* recv, const int64_t* recvcounts,
                       const int64_t* rdispls, int32_t elem_bytes);
  int32_t (*allreduce_i64)(void* ctx, int64_t* value, int32_t op);
} sp_comm;

typedef struct sp_ogs_mr sp_ogs_mr;

typedef struct {
  int32_t N;
  int32_t NlocalP, NlocalT;  /* local operator rows: with a positive member / all     */
  int32_t NhaloP, NhaloT;    /* halo operator rows: with a positive member here / all */
  int32_t Nshared;           /* (halo row, remote rank) pairs                         */
  int32_t gather_defined;    /* every group has exactly one positive member           */
  int32_t uploaded;          /* device operators exist                                */
  int64_t Ngather;           /* NlocalP + NhaloP                                      */
  int64_t NgatherGlobal;     /* Ngather summed over the ranks                         */
} sp_ogs_mr_info;

/* Exchange schedule of one transpose mode (ogsPairwise_t::data_t).  Send side: the
 * Nsend halo rows sendIds[] are packed into the send buffer, peer i of the send
 * list gets sendCounts[i]*k values from element sendOffsets[i]*k.  Receive side:
 * the halo buffer holds this rank's NrowsP rows first; peer j of the receive list
 * delivers recvCounts[j]*k values at element (NrowsP + recvOffsets[j])*k.  The
 * post-exchange gather reduces the Ncols = NrowsP + received columns into Nrows
 * rows (CSR postRowStarts/postColIds: this rank's row first, then the other ranks'
 * values in ascending rank order). */
typedef struct {
  int32_t Nsend, NrowsP, Nrows, Ncols;
  int32_t NranksSend, NranksRecv;
} sp_ogs_mr_sched;

/* Collective over comm.  h_ids[N] as sp_ogs_setup (signs written back with
 * unique).  upload == 0 builds the host half only (operators and schedules, no
 * device use); otherwise the operators are uploaded on `stream`. */
sp_status sp_ogs_mr_setup(int32_t N, int64_t* h_ids, sp_kind kind, int32_t unique,
                          const sp_comm* comm, int32_t upload, sp_stream_t stream,
                          sp_ogs_mr** out);
sp_status sp_ogs_mr_destroy(sp_ogs_mr* h);
sp_status sp_ogs_mr_info_get(const sp_ogs_mr* h, sp_ogs_mr_info* info);
/* Device operators (NULL before upload): which 0 = local, 1 = halo. */
const sp_ogs_plan* sp_ogs_mr_plan(const sp_ogs_mr* h, int32_t which);
/* Host CSR of the local (which 0) or halo (1) operator: op SP_TRANS -> T,
 * SP_NOTRANS -> N.  Arrays sized rows+1 and entries (either may be NULL). */
sp_status sp_ogs_mr_csr(const sp_ogs_mr* h, int32_t which, sp_transpose op,
                        int32_t* h_rowStarts, int32_t* h_colIds);
/* Schedule of one mode; any array may be NULL (sizes NranksSend, NranksRecv,
 * Nsend, Nrows + 1, Ncols). */
sp_status sp_ogs_mr_schedule(const sp_ogs_mr* h, sp_transpose mode, sp_ogs_mr_sched* s,
                             int32_t* h_sendRanks, int32_t* h_sendCounts,
                             int32_t* h_sendOffsets, int32_t* h_recvRanks,
                             int32_t* h_recvCounts, int32_t* h_recvOffsets,
                             int32_t* h_sendIds, int32_t* h_postRowStarts,
                             int32_t* h_postColIds);
/* Device halves of one exchange (ogsPairwise_t::DeviceStart / DeviceFinish without
 * the transport, ogsPairwise.cpp:106-156):
 *   start:  send[n*k + f] = halo[sendIds[n]*k + f]    (extract, ogsKernels.okl:167-177)
 *   finish: out[row*k + f] = op over the columns c of row, in CSR order, of
 *           halo[c*k + f]                              (the post-exchange gather)
 * halo holds Ncols*k values of the mode, send Nsend*k, out Nrows*k. */
sp_status sp_ogs_mr_exchange_start(const sp_ogs_mr* h, sp_type type, sp_transpose mode,
                                   int32_t k, const void* halo, void* send, sp_stream_t stream);
sp_status sp_ogs_mr_exchange_finish(const sp_ogs_mr* h, sp_type type, sp_op op,
                                    sp_transpose mode, int32_t k, const void* halo, void* out,
                                    sp_stream_t stream);

/* ---------------------------------------------------------------- batched instances
 * Many independent instances of uneven size in ONE persistent launch.  Instance i
 * owns x[i], r[i], p[i], Ap[i] (n[i] doubles), rdotr[i] (one double) and alpha[i],
 * and a node field q[i] with its own plan.  sp_batch_run performs, for every i,
 *   x += alpha p;  r -= alpha Ap;  rdotr = r.r      (values of sp_cg_update_f64;
 *                                                     r.r in its own fixed order)
 *   q <- GatherScatter(q, Add, Sym)                 (bits of sp_ogs_gather_scatter)
 * Arrays of device pointers are read at creation (host arrays); the plans must
 * outlive the batch and have warp chunks (every group <= 256 members).  Runs of one
 * batch must not overlap on the device (they share per-instance tickets). */
typedef struct sp_batch sp_batch;
sp_status sp_batch_create(int32_t ninst, const sp_ogs_plan* const* plans, const int64_t* n,
                          double* const* x, double* const* r, const double* const* p,
                          const double* const* Ap, double* const* rdotr, double* const* q,
                          const double* alpha, sp_stream_t stream, sp_batch** out);
/* FP32 storage: x, r, p, Ap, q in FP32 (x and r bit-identical to sp_cg_update_f32,
 * q to the FP32 gather+scatter); r.r from compensated FP32 tile partials summed in
 * FP64 into the FP64 rdotr[i]. */
sp_status sp_batch_create_f32(int32_t ninst, const sp_ogs_plan* const* plans, const int64_t* n,
                              float* const* x, float* const* r, const float* const* p,
                              const float* const* Ap, double* const* rdotr, float* const* q,
                              const double* alpha, sp_stream_t stream, sp_batch** out);
sp_status sp_batch_run(const sp_batch* b, sp_stream_t stream);
sp_status sp_batch_destroy(sp_batch* b);

/* ---------------------------------------------------------------- box mesh ids
 * Global node ids of a structured nx*ny*nz hex box of degree p on one rank, as
 * mesh_t::Setup produces them (SetupBoxHex3D libs/mesh/meshSetupBoxHex3D.cpp:87-130,
 * ConnectNodes libs/mesh/meshConnectNodes.cpp:43-81): id(l) = 1 + the smallest local
 * index l' = e'*Np + n' that sits on the same lattice point.  With perm_seed != 0 the
 * element slots are first permuted by a seeded Fisher-Yates shuffle (SplitMix64
 * stream), slot(e) = perm[e].  h_ids must hold nx*ny*nz*(p+1)^3 entries. */
sp_status sp_mesh_box_hex_ids(int32_t nx, int32_t ny, int32_t nz, int32_t p, uint64_t perm_seed,
                              int64_t* h_ids);
/* The same ids written into device memory d_ids by a kernel (one thread per local
 * node takes the minimum over the up to 8 element nodes on its lattice point);
 * synchronises `stream`. */
sp_status sp_mesh_box_hex_ids_device(int32_t nx, int32_t ny, int32_t nz, int32_t p,
                                     uint64_t perm_seed, int64_t* d_ids, sp_stream_t stream);
/* Ids of rank `rank` when `size` ranks each hold an nx*ny*nz box (mesh_t::SetupBoxHex3D
 * with the Factor3 / RankDecomp3 rank grid, libs/mesh/meshSetupBoxHex3D.cpp:44-53,
 * libs/core/rankDecomp.cpp; ConnectNodes across ranks numbers local node l of rank
 * r as r*E*Np + l): id = 1 + the smallest such global index on the same global
 * lattice point.  size == 1 gives sp_mesh_box_hex_ids. */
sp_status sp_mesh_box_hex_ids_rank(int32_t nx, int32_t ny, int32_t nz, int32_t p,
                                   uint64_t perm_seed, int32_t size, int32_t rank,
                                   int64_t* h_ids);

#ifdef __cplusplus
}
#endif
#endif /* SP_CAPI_H */
