// Device half of the multi-rank gather-scatter: the operators' upload, the send
// buffer packing (extract) and the post-exchange gather.
#include <algorithm>

#include "sp_ogs_mr.h"
#include "sp_ogs_plan.h"

namespace sp {
namespace {

// send[t] = halo[ids[t / k] * k + t % k]  (the reference's `extract`,
// libs/ogs/okl/ogsKernels.okl:167-177): consecutive threads write consecutive
// values; the reads follow the send order of the halo rows.
template <typename T>
__global__ void __launch_bounds__(256) k_ogs_extract(int64_t total, int32_t k,
                                                     const int32_t* __restrict__ ids,
                                                     const T* __restrict__ halo,
                                                     T* __restrict__ send) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
    const int64_t row = t / k;
    send[t] = halo[(int64_t)__ldg(ids + row) * k + (t - row * k)];
  }
}

template <typename T>
void launch_extract(const SpMrSched& x, int32_t k, const void* halo, void* send, cudaStream_t s) {
  const int64_t total = (int64_t)x.Nsend * k;
  const int64_t want = (total + 255) / 256;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sm_count() * 8));
  k_ogs_extract<T><<<grid, 256, 0, s>>>(total, k, x.d_sendIds, (const T*)halo, (T*)send);
}

sp_status check_handle(const sp_ogs_mr* h, sp_type type, sp_transpose mode, int32_t k,
                       const char* what) {
  if (!h) return fail(SP_ERR_INVALID_ARG, "%s: null handle", what);
  if (!h->op[0]) return fail(SP_ERR_INVALID_ARG, "%s: handle was set up without upload", what);
  if (type < SP_FLOAT || type > SP_INT64) return fail(SP_ERR_INVALID_ARG, "%s: bad type", what);
  if (mode < SP_SYM || mode > SP_TRANS) return fail(SP_ERR_INVALID_ARG, "%s: bad mode", what);
  if (k < 1) return fail(SP_ERR_INVALID_ARG, "%s: k must be >= 1", what);
  return SP_SUCCESS;
}

sp_status upload_ids(const std::vector<int32_t>& v, int32_t** d, cudaStream_t s) {
  SP_CUDA_TRY(cudaMalloc(d, std::max<size_t>(v.size(), 1) * sizeof(int32_t)));
  if (!v.empty())
    SP_CUDA_TRY(cudaMemcpyAsync(*d, v.data(), v.size() * sizeof(int32_t), cudaMemcpyHostToDevice, s));
  return SP_SUCCESS;
}

}  // namespace

sp_status mr_upload(sp_ogs_mr* h, cudaStream_t s) {
  SP_CUDA_TRY(cudaGetDevice(&h->device));
  const bool unsignedKind = (h->kind == SP_KIND_UNSIGNED);
  const int32_t rowsT[2] = {h->NlocalT, h->NhaloT}, rowsN[2] = {h->NlocalP, h->NhaloP};
  for (int part = 0; part < 2; ++part) {
    const std::vector<int32_t>* c = h->csr[part];
    sp_status st = sp_ogs_plan_create(h->N, rowsT[part], c[0].data(), c[1].data(), rowsN[part],
                                      unsignedKind ? nullptr : c[2].data(),
                                      unsignedKind ? nullptr : c[3].data(), (sp_stream_t)s,
                                      &h->op[part]);
    if (st) return st;
  }
  for (int mode = 0; mode < 3; ++mode) {
    SpMrSched& x = h->sched[mode];
    sp_status st = sp_ogs_plan_create(x.Ncols, x.Nrows, x.postRs.data(), x.postCi.data(), x.Nrows,
                                      nullptr, nullptr, (sp_stream_t)s, &x.post);
    if (st) return st;
    if ((st = upload_ids(x.sendIds, &x.d_sendIds, s))) return st;
  }
  SP_CUDA_TRY(cudaStreamSynchronize(s));
  return SP_SUCCESS;
}

void mr_free_device(sp_ogs_mr* h) {
  for (int part = 0; part < 2; ++part) {
    sp_ogs_plan_destroy(h->op[part]);
    h->op[part] = nullptr;
  }
  for (int mode = 0; mode < 3; ++mode) {
    sp_ogs_plan_destroy(h->sched[mode].post);
    h->sched[mode].post = nullptr;
    if (h->sched[mode].d_sendIds) cudaFree(h->sched[mode].d_sendIds);
    h->sched[mode].d_sendIds = nullptr;
  }
}

}  // namespace sp

using namespace sp;

extern "C" {

sp_status sp_ogs_mr_exchange_start(const sp_ogs_mr* h, sp_type type, sp_transpose mode,
                                   int32_t k, const void* halo, void* send, sp_stream_t stream) {
  sp_status st = check_handle(h, type, mode, k, "sp_ogs_mr_exchange_start");
  if (st) return st;
  const SpMrSched& x = h->sched[mode];
  if (x.Nsend == 0) return SP_SUCCESS;
  if (!halo || !send) return fail(SP_ERR_INVALID_ARG, "sp_ogs_mr_exchange_start: null buffer");
  const cudaStream_t s = as_cuda(stream);
  switch (type) {
    case SP_FLOAT: launch_extract<float>(x, k, halo, send, s); break;
    case SP_DOUBLE: launch_extract<double>(x, k, halo, send, s); break;
    case SP_INT32: launch_extract<int32_t>(x, k, halo, send, s); break;
    case SP_INT64: launch_extract<long long>(x, k, halo, send, s); break;
  }
  return check_launch("sp_ogs_mr_exchange_start");
}

sp_status sp_ogs_mr_exchange_finish(const sp_ogs_mr* h, sp_type type, sp_op op,
                                    sp_transpose mode, int32_t k, const void* halo, void* out,
                                    sp_stream_t stream) {
  sp_status st = check_handle(h, type, mode, k, "sp_ogs_mr_exchange_finish");
  if (st) return st;
  const SpMrSched& x = h->sched[mode];
  if (x.Nrows == 0) return SP_SUCCESS;
  if (!halo || !out) return fail(SP_ERR_INVALID_ARG, "sp_ogs_mr_exchange_finish: null buffer");
  return sp_ogs_gather(x.post, type, op, SP_SYM, k, out, halo, stream);
}

}  // extern "C"
