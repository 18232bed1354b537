// Persistent launch over an uneven batch: images of several geometries (each
// with its own patch grid, PSF size and FFT frame) processed by one kernel.
//
// The host builds a work list of (class, image, patch) items, largest frame
// first, and passes the per-class parameters by value.  A grid of 2-CTA
// clusters (one CTA per SM) walks the list statically: cluster c takes items
// c, c + #clusters, ...; both CTAs of a cluster derive the same sequence, so
// no queue, atomic or wait is involved.  Each item runs eff_patch for its
// frame size, which ends on a cluster barrier before the next item starts.
#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "eff_internal.h"
#include "eff_launch.cuh"
#include "../../include/vmbd_eff.h"

namespace eff {

constexpr int kMaxClasses = 8;
constexpr int kBatchThreads = 512;

// Defined with the plan (eff_capi.cu): the plan's kernel parameters with no
// data pointers, its frame edge, and its patch count.
int plan_params(const EffPlan* plan, Params* P, int* N);
int plan_patches(const EffPlan* plan);

struct ClassTable {
  int n;
  int N[kMaxClasses];
  Params P[kMaxClasses];
};

struct Item {
  int cls, b, k, pad;
};

// One patch of one frame size as a separate (not inlined) function: the
// persistent kernel calls one per item, and each is register-allocated and
// compiled on its own instead of as one very large kernel body.
template <int N, int OP>
__device__ __noinline__ void batch_patch(const Params& P, int k, long long b, float2* smem, int cta, int ncta) {
  eff_patch<N, OP, 2>(P, k, b, smem, cta, ncta);
}

template <int OP>
__global__ void __launch_bounds__(kBatchThreads) eff_persistent(const ClassTable T, const Item* __restrict__ items,
                                                                int n_items) {
  extern __shared__ __align__(16) float2 smem[];
  const int rank = (int)cg::this_cluster().block_rank();
  const int cid = blockIdx.x / 2, ncl = gridDim.x / 2;
  for (int i = cid; i < n_items; i += ncl) {
    const Item it = items[i];
    const Params& P = T.P[it.cls];
    const int K = P.csf0 * P.csf1;
    switch (T.N[it.cls]) {
      case 256: batch_patch<256, OP>(P, it.k, it.b, smem, 2 * it.k + rank, 2 * K); break;
      case 192: batch_patch<192, OP>(P, it.k, it.b, smem, 2 * it.k + rank, 2 * K); break;
      case 128: batch_patch<128, OP>(P, it.k, it.b, smem, 2 * it.k + rank, 2 * K); break;
      default: batch_patch<64, OP>(P, it.k, it.b, smem, 2 * it.k + rank, 2 * K); break;
    }
  }
}

template <int OP>
cudaError_t launch_persistent(const ClassTable& T, const Item* items, int n_items, int grid, size_t smem,
                              cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(eff_persistent<OP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kBatchThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = cudaLaunchKernelEx(&cfg, eff_persistent<OP>, T, items, n_items);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

}  // namespace eff

// Batch of plans: per class the plan, its image count and its parameter
// template; the device work list.
struct EffBatch {
  int n;
  const EffPlan* plans[eff::kMaxClasses];
  int counts[eff::kMaxClasses];
  eff::Item* items;
  int n_items;
  int grid;
  int device;  // of every plan and of the work list
};

namespace {

int fail(int code, const std::string& msg) { return eff::set_error(code, msg); }

}  // namespace

extern "C" {

int eff_batch_create(const EffPlan* const* plans, const int* counts, int n_classes, EffBatch** out) {
  if (!plans || !counts || !out || n_classes < 1) return fail(EFF_ERR_INVALID, "null argument");
  *out = nullptr;
  if (n_classes > eff::kMaxClasses)
    return fail(EFF_ERR_UNSUPPORTED, "at most " + std::to_string(eff::kMaxClasses) + " geometries per batch");
  EffBatch B;
  std::memset(&B, 0, sizeof(B));
  B.n = n_classes;
  std::vector<eff::Item> items;
  std::vector<std::pair<int, int>> order;  // (frame, class)
  for (int c = 0; c < n_classes; ++c) {
    if (!plans[c] || counts[c] < 1) return fail(EFF_ERR_INVALID, "bad plan or count");
    if (int s = eff::check_plan_device(plans[c])) return s;
    if (eff::plan_deterministic(plans[c]))  // the persistent kernel overlap-adds with atomics
      return fail(EFF_ERR_UNSUPPORTED, "deterministic plans are not supported in a persistent batch");
    B.plans[c] = plans[c];
    B.counts[c] = counts[c];
    int n = 0;
    eff_plan_frame(plans[c], &n);
    if (n == 512)  // its patches need clusters of 4-8 CTAs, the persistent grid has pairs
      return fail(EFF_ERR_UNSUPPORTED, "frame 512 is not supported in a persistent batch");
    order.push_back({-n, c});
  }
  std::stable_sort(order.begin(), order.end());
  for (auto& oc : order) {
    const int c = oc.second;
    const int K = eff::plan_patches(plans[c]);
    for (int b = 0; b < counts[c]; ++b)
      for (int k = 0; k < K; ++k) items.push_back({c, b, k, 0});
  }
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return fail(EFF_ERR_CUDA, std::string("device query: ") + cudaGetErrorString(e));
  B.device = dev;
  B.grid = std::max(2, (sms / 2) * 2);
  B.n_items = (int)items.size();
  e = cudaMalloc(&B.items, sizeof(eff::Item) * items.size());
  if (e != cudaSuccess) return fail(EFF_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  e = cudaMemcpy(B.items, items.data(), sizeof(eff::Item) * items.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(B.items);
    return fail(EFF_ERR_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
  }
  EffBatch* p = new (std::nothrow) EffBatch(B);
  if (!p) {
    cudaFree(B.items);
    return fail(EFF_ERR_INVALID, "out of host memory");
  }
  *out = p;
  return EFF_OK;
}

int eff_batch_destroy(EffBatch* batch) {
  if (!batch) return EFF_OK;
  cudaFree(batch->items);
  delete batch;
  return EFF_OK;
}

int eff_batch_items(const EffBatch* batch) { return batch ? batch->n_items : 0; }

}  // extern "C"

namespace eff {

// Fill a class table from the plans and the per-class pointers, size shared
// memory, clear atomically accumulated outputs, launch.
int batch_run(const EffBatch* B, int op, const float* const* x, const float* const* f, const float* const* y,
              const float* const* y_obs, const void* const* spec0, const void* const* spec1, float* const* out0,
              float* const* out1, void* const* a_out, void* const* b_out, double* const* loss, void* stream) {
  if (!B) return set_error(EFF_ERR_INVALID, "null batch");
  // the plans' tables and the work list live on the batch's device
  for (int c = 0; c < B->n; ++c)
    if (int s = check_plan_device(B->plans[c])) return s;
  ClassTable T;
  std::memset(&T, 0, sizeof(T));
  T.n = B->n;
  size_t smem = 0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  for (int c = 0; c < B->n; ++c) {
    Params P;
    if (int s = plan_params(B->plans[c], &P, &T.N[c])) return s;
    const int batch = B->counts[c];
    if (op == OP_FWD_BOTH) {
      if (!x || !f || !y || !x[c] || !f[c] || !y[c]) return set_error(EFF_ERR_INVALID, "null argument");
      P.x = x[c];
      P.f = f[c];
      P.out0 = const_cast<float*>(y[c]);
      P.out0_bs = P.y_bs;
      P.a_out = a_out ? static_cast<float2*>(a_out[c]) : nullptr;
      P.b_out = b_out ? static_cast<float2*>(b_out[c]) : nullptr;
      if (y_obs) {  // residual forward: the output ends as EFF - y_obs
        if (!y_obs[c] || y_obs[c] == y[c]) return set_error(EFF_ERR_INVALID, "bad y_obs");
        P.sub = y_obs[c];
      }
      cudaError_t e = cudaMemsetAsync(P.out0, 0, sizeof(float) * P.y_bs * batch, st);
      if (e != cudaSuccess) return set_error(EFF_ERR_CUDA, std::string("memset: ") + cudaGetErrorString(e));
    } else {
      if (!y || !y[c]) return set_error(EFF_ERR_INVALID, "null y");
      P.y = y[c];
      P.y_obs = y_obs ? y_obs[c] : nullptr;
      P.b0 = spec0 ? static_cast<const float2*>(spec0[c]) : nullptr;
      P.b1 = spec1 ? static_cast<const float2*>(spec1[c]) : nullptr;
      P.out0 = out0 ? out0[c] : nullptr;
      P.out1 = out1 ? out1[c] : nullptr;
      P.loss = loss ? loss[c] : nullptr;
      P.loss_y = P.y_obs ? 0 : 1;  // no y_obs: y is the residual
      P.out0_bs = P.x_bs;
      P.out1_bs = P.f_bs;
      if (!P.out0 && !P.out1) return set_error(EFF_ERR_INVALID, "no adjoint output");
      if ((P.out0 && !P.b0) || (P.out1 && !P.b1)) return set_error(EFF_ERR_INVALID, "missing spectrum");
      cudaError_t e = cudaSuccess;
      if (P.out0) e = cudaMemsetAsync(P.out0, 0, sizeof(float) * P.x_bs * batch, st);
      if (e == cudaSuccess && P.loss) e = cudaMemsetAsync(P.loss, 0, sizeof(double) * batch, st);
      if (e != cudaSuccess) return set_error(EFF_ERR_CUDA, std::string("memset: ") + cudaGetErrorString(e));
    }
    T.P[c] = P;
    smem = std::max(smem, smem_bytes(T.N[c], op, P, kBatchThreads, 2));
  }
  if (smem > 227u * 1024u)
    return set_error(EFF_ERR_UNSUPPORTED, "a batch member needs " + std::to_string(smem) + " bytes of shared memory");
  cudaError_t e = op == OP_FWD_BOTH ? launch_persistent<OP_FWD_BOTH>(T, B->items, B->n_items, B->grid, smem, st)
                                    : launch_persistent<OP_ADJ>(T, B->items, B->n_items, B->grid, smem, st);
  if (e != cudaSuccess) return set_error(EFF_ERR_CUDA, std::string("persistent launch: ") + cudaGetErrorString(e));
  return EFF_OK;
}

}  // namespace eff

extern "C" {

int eff_batch_forward_both(const EffBatch* batch, const float* const* x, const float* const* f, float* const* y,
                           void* const* xhat_out, void* const* fhat_out, void* stream) {
  return eff::batch_run(batch, eff::OP_FWD_BOTH, x, f, y, nullptr, nullptr, nullptr, nullptr, nullptr, xhat_out,
                        fhat_out, nullptr, stream);
}

int eff_batch_forward_residual(const EffBatch* batch, const float* const* x, const float* const* f,
                               const float* const* y_obs, float* const* r, void* const* xhat_out,
                               void* const* fhat_out, void* stream) {
  if (!y_obs) return eff::set_error(EFF_ERR_INVALID, "null y_obs");
  return eff::batch_run(batch, eff::OP_FWD_BOTH, x, f, r, y_obs, nullptr, nullptr, nullptr, nullptr, xhat_out,
                        fhat_out, nullptr, stream);
}

int eff_batch_adjoint_residual(const EffBatch* batch, const float* const* y, const float* const* y_obs,
                               const void* const* fhat, const void* const* xhat, float* const* gx,
                               float* const* gf, double* const* loss, void* stream) {
  return eff::batch_run(batch, eff::OP_ADJ, nullptr, nullptr, y, y_obs, fhat, xhat, gx, gf, nullptr, nullptr,
                        loss, stream);
}

}  // extern "C"
