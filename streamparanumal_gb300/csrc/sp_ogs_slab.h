// Lane-row slab gathers (kernel 7): launch entry points used by the ogs dispatch.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace sp {

// The slab layout of one walk on the device (build_slabs; codes, tabs and td from
// compress_slabs, or null with shift 0; rcodes, rtabs and rtd the row words' codes
// from compress_slab_rows, or null).
struct SlabArgs {
  const int4* slabs;
  int32_t nslabs;
  const int32_t* ids;
  const int32_t* rows;
  const uint16_t* codes;
  const int32_t* tabs;
  const int2* td;
  int shift;
  const uint16_t* rcodes;
  const int32_t* rtabs;
  const int2* rtd;
};

// One launch over the slabs of a walk: MODE 1 gathers gv[row] = op over the row's
// members of v (rows from `rows`); MODE 0 writes that result back to every member
// of v in place (gather+scatter, Sym), `rows` unused.
template <typename T, int OP, int MODE>
void launch_slabs(const SlabArgs& a, T* v, T* gv, cudaStream_t s);

}  // namespace sp
