/*
 * sp_oracle.h -- CPU restatement of streamParanumal's streaming hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the GPU kernels are
 * compared against (and the timed CPU baseline of bench.py).  Nothing in the
 * product links, loads or calls it.
 *
 * Each function states which reference file:line it restates.  Arithmetic is
 * written so that the rounding is explicit: the library is compiled with
 * -ffp-contract=off and every fused multiply-add is a call to fma().
 * `fmad` arguments select the reference's CUDA-mode contraction (--fmad=true,
 * libs/core/platformProperties.cpp:76) when non-zero, or the Serial-mode
 * separate multiply and add when zero.
 */
#ifndef SP_ORACLE_H
#define SP_ORACLE_H

#include <stdint.h>

/* ---- BS1..BS5 (OCCA Serial semantics of the OKL kernels) ---- */
void or_bs1(int64_t n, const double* a, double* b);                                  /* bs1.okl:31-33 */
void or_bs2(int64_t n, double alpha, const double* x, double beta, double* y, int fmad); /* bs2.okl:33-35 */
void or_bs2_f32(int64_t n, float alpha, const float* x, float beta, float* y, int fmad);
void or_bs3_1(int bs, int nblocks, int64_t n, const double* a, double* partial, int fmad); /* bs3.okl:27-64 */
void or_bs4_1(int bs, int nblocks, int64_t n, const double* a, const double* b, double* partial, int fmad); /* bs4.okl:27-65 */
void or_bs5_1(int bs, int nblocks, int64_t n, const double* Ap, double alpha, double* r, double* partial, int fmad); /* bs5.okl:27-67 */
void or_finish(int bs, int nblocks, const double* partial, double* out);             /* bs3.okl:66-102 */

/* Accurate references (double-double accumulation) for the tolerance checks. */
double or_dot_dd(int64_t n, const double* a, const double* b);
double or_dot_dd_f32(int64_t n, const float* a, const float* b);
/* x += alpha p; r -= alpha Ap (fma forms); returns sum r*r in double-double. */
double or_cg_update(int64_t n, double alpha, const double* p, const double* Ap, double* x, double* r);
double or_cg_update_f32(int64_t n, float alpha, const float* p, const float* Ap, float* x, float* r);

/* ---- mesh ids: reference algorithm (libs/mesh/meshSetupBoxHex3D.cpp:87-130,
 * libs/mesh/meshConnectNodes.cpp:43-81): start from 1 + local index and repeatedly
 * take the smaller id across every pair of coincident face nodes of neighbouring
 * elements until nothing changes.  perm_seed != 0 permutes element slots with a
 * SplitMix64-driven Fisher-Yates shuffle. */
int or_box_hex_ids(int nx, int ny, int nz, int p, uint64_t perm_seed, int64_t* ids);

/* ---- ogs setup at one rank (libs/ogs/ogsSetup.cpp:87-290, 492-579) ----
 * Fills the T and N CSR; arrays must hold N entries (colIds) and N+1 (rowStarts).
 * Returns 0 on success.  kind: 0 Unsigned, 1 Signed, 2 Halo.  ids modified when
 * unique. */
int or_ogs_setup(int32_t N, int64_t* ids, int kind, int unique,
                 int32_t* NrowsT, int32_t* rowStartsT, int32_t* colIdsT,
                 int32_t* NrowsN, int32_t* rowStartsN, int32_t* colIdsN);

/* ---- ogsOperator host loops (libs/ogs/ogsOperator.cpp:61-114, 223-267, 340-409) ----
 * type: 0 float, 1 double, 2 int32, 3 int64.  op: 0 add, 1 mul, 2 max, 3 min. */
void or_ogs_gather(int type, int op, int32_t Nrows, const int32_t* rowStarts, const int32_t* colIds,
                   int k, void* gv, const void* v);
void or_ogs_scatter(int type, int32_t Nrows, const int32_t* rowStarts, const int32_t* colIds,
                    int k, void* v, const void* gv);
void or_ogs_gather_scatter(int type, int op, int32_t Nrows,
                           const int32_t* gRowStarts, const int32_t* gColIds,
                           const int32_t* sRowStarts, const int32_t* sColIds, int k, void* v);

/* Seeded uniform[-1,1) doubles: SplitMix64 stream, u = (z >> 11) * 2^-53, x = 2u - 1. */
void or_fill_uniform(int64_t n, uint64_t seed, double* x);

#endif
