// C ABI of the EFF operator (declared in include/vmbd_eff.h).
//
// Plan creation validates the geometry as OlaGPU.__init__ does
// (olaGPU.py:95-168), uploads the separable window factors and the FP64-built
// twiddle table, and picks the FFT frame.  The compute entry points only
// enqueue work on the caller's stream (a clear of atomically accumulated
// outputs + one kernel) and allocate nothing.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "eff_internal.h"
#include "eff_launch.cuh"
#include "eff_ola.h"
#include "../../include/vmbd_eff.h"

namespace eff {
int plan_params(const EffPlan* plan, Params* P, int* N);
int plan_patches(const EffPlan* plan);
cudaError_t launch_project(float* f, int K, int n, int mode, cudaStream_t st);
cudaError_t launch_basis_project(const float* fs, const float* basis, float* w, int nb, int n,
                                 cudaStream_t st);
cudaError_t launch_edgetaper(float* im, int rows, int cols, const float* wy, int hy, const float* wx,
                             int hx, int batch, cudaStream_t st);
cudaError_t launch_dots3(const float* a, const float* ap, long long na, const float* b, const float* bp,
                         long long nb, double* out, bool zeroed, cudaStream_t st);
cudaError_t launch_pg_step(float* f, const float* g, float* fp, float* gp, int K, int n, const double* dots,
                           int mode, float* state, float* zero_f, long long zero_n, cudaStream_t st);
cudaError_t launch_max_nonneg(const float* a, long long n, unsigned* out_bits, cudaStream_t st);
cudaError_t launch_mu_update(float* x, const float* num, const float* den, float tol, int rows, int cols,
                             int b0, int b1, const unsigned* num_max_bits, float floor_rel, unsigned* xmax_bits,
                             bool zeroed, float* zero_f, long long zero_n, cudaStream_t st);
}  // namespace eff

struct EffPlan {
  EffGeom g;
  int N;
  int K;
  int sy[2], off[2], E[2];
  int threads;   // per CTA when one CTA handles a patch
  int threads2;  // per CTA of a 2-CTA cluster (frame 512: of a clw-CTA cluster)
  int clw;       // frame 512: CTAs per patch (4, or 8 when a quarter frame does not fit)
  int num_sms;
  int device;
  float2* win0;
  float2* win1;
  float2* tw;   // twiddle table [N], followed in the same allocation by
  float* lap;   // the difference-filter spectrum 4 sin^2(pi k / N) [N]
  int* err;     // and the device error word
  bool det;            // EFF_GEOM_DETERMINISTIC: tile stores + ola_gather instead of atomics
  float* tiles;        // deterministic: one image's patch tiles, K * max(E0 E1, sw0 sw1) floats
  double* loss_part;   // deterministic: one image's per-CTA loss shares, K * 8 doubles
};

namespace {

thread_local std::string g_last_error;
constexpr size_t kSmemLimit = 227u * 1024u;
// 0: choose per call; 1: one CTA per patch; 2: a 2-CTA cluster per patch.
std::atomic<int> g_cluster_mode{0};
// 1 (default): kernels whose first operand is the image copy each CTA's rows
// of the patch window into shared memory with one tensor-engine copy where
// the geometry allows (see image_tile); 0: every lane loads its values.
std::atomic<int> g_image_tile{1};
// Cached spectra staged in shared memory (bulk copies at kernel start,
// where they fit) or read from global memory: 2 (default) staged for the
// deconvolution only, whose spectra usually come from HBM (512^2: 22.5 vs
// 25.6 us), read for the rest -- a loss/gradient step's adjoint finds its
// spectra in L2, just written by the forward (step 35.7 vs 36.8 us
// staged); 1 staged for every kernel that multiplies by one; 0 never.
std::atomic<int> g_stage_spectra{2};

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(EFF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Frame edges chosen automatically (ascending): the powers of two.  The
// 192 frame (24 x 8 mixed radix) is compiled too but only used on request:
// its 24 values per lane make each lane's dependent chain ~1.5x longer, which
// costs more than its ~45% less arithmetic saves on latency-bound single
// images; batches that fill the GPU can gain (the batch autotuner tries it).
constexpr int kFrames[] = {64, 128, 256, 512};
int frame_ok(int n) { return n == 64 || n == 128 || n == 192 || n == 256 || n == 512; }

eff::Params base_params(const EffPlan* p) {
  eff::Params P;
  std::memset(&P, 0, sizeof(P));
  const EffGeom& g = p->g;
  P.sx0 = g.sx[0]; P.sx1 = g.sx[1];
  P.sf0 = g.sf[0]; P.sf1 = g.sf[1];
  P.csf0 = g.csf[0]; P.csf1 = g.csf[1];
  P.sw0 = g.sw[0]; P.sw1 = g.sw[1];
  P.hop0 = g.hop[0]; P.hop1 = g.hop[1];
  P.sy0 = p->sy[0]; P.sy1 = p->sy[1];
  P.off0 = p->off[0]; P.off1 = p->off[1];
  P.E0 = p->E[0]; P.E1 = p->E[1];
  P.lo0 = 0; P.hi0 = p->E[0]; P.lo1 = 0; P.hi1 = p->E[1];
  P.win0 = p->win0;
  P.win1 = p->win1;
  P.tw = p->tw;
  P.lap = p->lap;
  P.err = p->err;
  P.x_bs = (long long)g.sx[0] * g.sx[1];
  P.f_bs = (long long)p->K * g.sf[0] * g.sf[1];
  P.y_bs = (long long)p->sy[0] * p->sy[1];
  P.spec_bs = (long long)p->K * (p->N / 2 + 1) * p->N;
  return P;
}

int launch_kernel(const EffPlan* p, int op, const eff::Params& P, int batch, int CL, int threads, size_t smem,
                  cudaStream_t st, const CUtensorMap* xmap = nullptr) {
  cudaError_t e;
  switch (p->N) {
    case 64: e = eff::launch_n64(op, CL, P, p->K, batch, threads, smem, st, xmap); break;
    case 128: e = eff::launch_n128(op, CL, P, p->K, batch, threads, smem, st, xmap); break;
    case 192: e = eff::launch_n192(op, CL, P, p->K, batch, threads, smem, st, xmap); break;
    case 256: e = eff::launch_n256(op, CL, P, p->K, batch, threads, smem, st, xmap); break;
    case 512: e = eff::launch_n512(op, CL, P, p->K, batch, threads, smem, st, xmap); break;
    default: return fail(EFF_ERR_UNSUPPORTED, "frame size");
  }
  if (e != cudaSuccess)
    return cuda_fail(e, ("kernel launch (frame " + std::to_string(p->N) + ", op " + std::to_string(op) + ", " +
                         std::to_string(CL) + " CTA(s) per patch, " + std::to_string(threads) + " threads, " +
                         std::to_string(smem) + " B shared)")
                            .c_str());
  return EFF_OK;
}

// Calls whose output is overlap-added (forwards; the image adjoint and the
// loss; the deconvolution's image estimate) run, on a deterministic plan, as
// the kernel storing patch tiles + ola_gather.
bool deterministic_ola(const EffPlan* p, int op, const eff::Params& P) {
  if (!p->det) return false;
  if (op == eff::OP_FWD_IMAGE || op == eff::OP_FWD_PSF || op == eff::OP_FWD_BOTH) return true;
  if (op == eff::OP_ADJ) return P.out0 || P.loss;
  if (op == eff::OP_DECONV) return P.out0;
  return false;
}

// Clear the outputs the kernel described by P accumulates into (a and b,
// nullable) with the zero kernel, and launch that kernel right behind it
// (P.pdl = 2): its transforms run beside the clear, and it waits for the
// clear before its output phase.  Saves the separate memset's dependency
// (about 2 us per call in a captured graph).  A deterministic plan stores
// its outputs whole: nothing to clear.
int clear_before(const EffPlan* p, eff::Params& P, void* a, size_t abytes, void* b, size_t bbytes,
                 cudaStream_t st) {
  if (p->det || (!a && !b)) return EFF_OK;
  eff::ZeroArgs Z;
  Z.p[0] = a;
  Z.bytes[0] = a ? (long long)abytes : 0;
  Z.p[1] = b;
  Z.bytes[1] = b ? (long long)bbytes : 0;
  cudaError_t e = eff::launch_zero(Z, p->num_sms, st);
  if (e != cudaSuccess) return cuda_fail(e, "clearing an output");
  P.pdl = 2;
  return EFF_OK;
}

// The parameters of image b of a batch, for a launch over that image alone.
eff::Params image_params(const eff::Params& P, long long b) {
  eff::Params Q = P;
  auto adv = [b](auto* ptr, long long stride) { return ptr ? ptr + b * stride : ptr; };
  Q.x = adv(P.x, P.x_bs);
  Q.f = adv(P.f, P.f_bs);
  Q.y = adv(P.y, P.y_bs);
  Q.y_obs = adv(P.y_obs, P.y_bs);
  Q.mask = adv(P.mask, P.y_bs);
  Q.sub = adv(P.sub, P.y_bs);
  Q.b0 = adv(P.b0, P.spec_bs);
  Q.b1 = adv(P.b1, P.spec_bs);
  Q.a_out = adv(P.a_out, P.spec_bs);
  Q.b_out = adv(P.b_out, P.spec_bs);
  Q.out0 = adv(P.out0, P.out0_bs);
  Q.out1 = adv(P.out1, P.out1_bs);
  Q.loss = adv(P.loss, 1);
  Q.pf = adv(P.pf, P.pf_bytes);
  return Q;
}

// Deterministic overlap-add: per image (the plan holds one image's tiles),
// the kernel storing its patch tiles, then the gather summing them in a
// fixed order (and subtracting the observation / summing the loss shares).
int run_deterministic(const EffPlan* p, int op, const eff::Params& P, int batch, int CL, int threads, size_t smem,
                      cudaStream_t st) {
  const bool fwd = op == eff::OP_FWD_IMAGE || op == eff::OP_FWD_PSF || op == eff::OP_FWD_BOTH;
  for (int b = 0; b < batch; ++b) {
    eff::Params Q = image_params(P, b);
    const float* sub = Q.sub;
    Q.sub = nullptr;  // the gather subtracts it
    Q.tiles = p->tiles;
    Q.loss_part = (op == eff::OP_ADJ && Q.loss) ? p->loss_part : nullptr;
    if (int s = launch_kernel(p, op, Q, 1, CL, threads, smem, st)) return s;
    eff::GatherArgs A;
    std::memset(&A, 0, sizeof(A));
    A.tiles = p->tiles;
    A.csf0 = p->g.csf[0];
    A.csf1 = p->g.csf[1];
    A.hop0 = p->g.hop[0];
    A.hop1 = p->g.hop[1];
    if (fwd) {
      A.th = p->E[0];
      A.tw = p->E[1];
      A.off0 = p->off[0];
      A.off1 = p->off[1];
      A.rows = p->sy[0];
      A.cols = p->sy[1];
      A.sub = sub;
    } else {
      A.th = p->g.sw[0];
      A.tw = p->g.sw[1];
      A.rows = Q.out0 ? p->g.sx[0] : 0;
      A.cols = Q.out0 ? p->g.sx[1] : 0;
    }
    A.out = Q.out0;
    if (Q.loss_part) {
      A.loss_part = Q.loss_part;
      A.nparts = p->K * CL;
      A.loss = Q.loss;
    }
    cudaError_t e = eff::launch_ola_gather(A, p->num_sms, st);
    if (e != cudaSuccess) return cuda_fail(e, "overlap-add gather launch");
  }
  return EFF_OK;
}

// cuTensorMapEncodeTiled, looked up once through the runtime (no link
// dependency on the driver library).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = []() -> EncodeTiledFn {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    (void)cudaGetLastError();
    return reinterpret_cast<EncodeTiledFn>(f);
  }();
  return fn;
}

// The image tile of kernels whose operand A is the image: a tensor map over
// x as [batch][sx0][sx1] floats and, in P, the box each CTA copies (tile_w
// columns: sw1 rounded up to 4; tile_rows: the rows of the image units one
// CTA transforms -- 2 NG of them when the cluster takes all units in one
// round, else the whole window).  Only where the copy is well formed: x
// 16-byte aligned, image rows and the patch hop multiples of 4 floats (so
// that every box starts on a 16-byte boundary), box sides <= 256.  False:
// the kernel loads its values itself.
bool image_tile(const EffPlan* p, int op, eff::Params& P, int batch, int CL, int threads, CUtensorMap* map) {
  P.tile_rows = P.tile_w = 0;
  if (!g_image_tile.load() || eff::opnd_a(op) != eff::OPND_IMAGE || !P.x || p->det) return false;
  const EffGeom& g = p->g;
  if ((reinterpret_cast<unsigned long long>(P.x) & 15ull) || (g.sx[1] & 3) || (g.hop[1] & 3)) return false;
  const int G = p->N / eff::lane_values(p->N), NG = threads / G, NW = CL * NG;
  const int nA = (g.sw[0] + 1) / 2;
  const int rows = (CL > 1 && nA <= NW) ? std::min(2 * NG, eff::even_up(g.sw[0])) : eff::even_up(g.sw[0]);
  const int w = (g.sw[1] + 3) & ~3;
  if (rows > 256 || w > 256) return false;
  EncodeTiledFn enc = encode_tiled();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)g.sx[1], (cuuint64_t)g.sx[0], (cuuint64_t)batch};
  const cuuint64_t strides[2] = {(cuuint64_t)g.sx[1] * sizeof(float), (cuuint64_t)g.sx[0] * g.sx[1] * sizeof(float)};
  const cuuint32_t box[3] = {(cuuint32_t)w, (cuuint32_t)rows, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  if (enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(P.x), dims, strides, box, estr,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  P.tile_rows = rows;
  P.tile_w = w;
  return true;
}

int run(const EffPlan* p, int op, const eff::Params& P0, int batch, void* stream) {
  eff::Params P = P0;
  P.stage_spec = 0;
  const size_t smem1 = eff::smem_bytes(p->N, op, P, p->threads, 1);
  const size_t smem2 = eff::smem_bytes(p->N, op, P, p->threads2, 2);
  // A 2-CTA cluster per patch when one CTA's frame does not fit, or when the
  // doubled grid still fits in one wave (more SMs on a small launch).
  // Frame 512 always runs on its clw-CTA clusters.
  const int mode = g_cluster_mode.load();
  int CL;
  if (p->N == 512) CL = p->clw;
  else if (smem1 > kSmemLimit) CL = 2;
  else if (mode == 1) CL = 1;
  else if (mode == 2) CL = 2;
  else CL = (2LL * p->K * batch <= p->num_sms) ? 2 : 1;
  const int threads = CL == 1 ? p->threads : p->threads2;
  // Kernels that multiply by cached spectra stage their columns of them in
  // shared memory where that still fits.
  if (op == eff::OP_ADJ || op == eff::OP_FWD_IMAGE || op == eff::OP_FWD_PSF || op == eff::OP_DECONV) {
    P.stage_spec = 1;
    const int mode = g_stage_spectra.load();
    if (eff::smem_bytes(p->N, op, P, threads, CL) > kSmemLimit || mode == 0 ||
        (mode == 2 && op != eff::OP_DECONV))
      P.stage_spec = 0;
  }
  CUtensorMap xmap;
  const bool tile = image_tile(p, op, P, batch, CL, threads, &xmap);
  if (tile && eff::smem_bytes(p->N, op, P, threads, CL) > kSmemLimit) P.tile_rows = P.tile_w = 0;
  const size_t smem = eff::smem_bytes(p->N, op, P, threads, CL);
  if (smem > kSmemLimit)
    return fail(EFF_ERR_UNSUPPORTED, "frame needs " + std::to_string(smem) + " bytes of shared memory");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (deterministic_ola(p, op, P)) return run_deterministic(p, op, P, batch, CL, threads, smem, st);
  return launch_kernel(p, op, P, batch, CL, threads, smem, st, P.tile_rows > 0 ? &xmap : nullptr);
}

// The plan's tables live on the device that was current at eff_plan_create;
// a kernel launched while another device is current would read them through
// addresses of that other device.  Refused before any memset or launch.
int check_device(const EffPlan* p) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev != p->device)
    return fail(EFF_ERR_INVALID, "plan was created on device " + std::to_string(p->device) + " but device " +
                                     std::to_string(dev) + " is current");
  return EFF_OK;
}

int check_plan(const EffPlan* p, int batch) {
  if (!p) return fail(EFF_ERR_INVALID, "null plan");
  if (batch < 1 || batch > 65535) return fail(EFF_ERR_INVALID, "batch must be in [1, 65535]");
  return check_device(p);
}

// zeroed: gx and loss were already zeroed on the stream (by the fused forward).
int adjoint_impl(const EffPlan* plan, const float* y, const float* y_obs, const void* fhat,
                 const void* xhat, float* gx, float* gf, double* loss, int adj_mode, int batch,
                 void* stream, const float* mask = nullptr, bool zeroed = false, bool loss_y = false,
                 bool after_forward = false) {
  if (int s = check_plan(plan, batch)) return s;
  if (!y || (!gx && !gf)) return fail(EFF_ERR_INVALID, "null argument");
  if (gx && !fhat) return fail(EFF_ERR_INVALID, "image adjoint needs the PSF spectrum");
  if (gf && !xhat) return fail(EFF_ERR_INVALID, "PSF adjoint needs the image spectrum");
  if (adj_mode != EFF_ADJ_EXACT && adj_mode != EFF_ADJ_REFERENCE)
    return fail(EFF_ERR_INVALID, "adj_mode");
  if (adj_mode == EFF_ADJ_REFERENCE && plan->g.mode == EFF_MODE_FULL)
    return fail(EFF_ERR_INVALID, "Not a valid mode!");  // olaGPU.py:285-286
  eff::Params P = base_params(plan);
  P.y = y;
  P.y_obs = y_obs;
  P.mask = mask;
  P.b0 = static_cast<const float2*>(fhat);
  P.b1 = static_cast<const float2*>(xhat);
  P.out0 = gx;
  P.out1 = gf;
  P.loss = loss;
  P.loss_y = loss_y ? 1 : 0;
  P.pdl = after_forward ? 1 : 0;
  P.out0_bs = P.x_bs;
  P.out1_bs = P.f_bs;
  if (adj_mode == EFF_ADJ_REFERENCE) {
    // chop_pad_GPU at offset `off`, extent sw (olaGPU.py:276-286).
    P.lo0 = plan->off[0];
    P.hi0 = plan->off[0] + plan->g.sw[0] < plan->E[0] ? plan->off[0] + plan->g.sw[0] : plan->E[0];
    P.lo1 = plan->off[1];
    P.hi1 = plan->off[1] + plan->g.sw[1] < plan->E[1] ? plan->off[1] + plan->g.sw[1] : plan->E[1];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (!zeroed) {
    if (int s = clear_before(plan, P, gx, sizeof(float) * P.x_bs * batch, loss, sizeof(double) * batch, st))
      return s;
  }
  return run(plan, eff::OP_ADJ, P, batch, stream);
}

// Workspace of the fused loss/gradient step: the two cached spectra and the
// forward output, each 256-byte aligned.
struct Workspace {
  size_t xhat, fhat, y, total;
};

Workspace workspace_layout(const EffPlan* p, int batch) {
  auto up = [](size_t v) { return (v + 255) & ~size_t(255); };
  const size_t spec = sizeof(float2) * (size_t)p->K * (p->N / 2 + 1) * p->N * batch;
  const size_t ybytes = sizeof(float) * (size_t)p->sy[0] * p->sy[1] * batch;
  Workspace w;
  w.xhat = 0;
  w.fhat = up(spec);
  w.y = w.fhat + up(spec);
  w.total = w.y + up(ybytes);
  return w;
}

// Forward from raw (x, f) leaving both spectra in the workspace, then both
// adjoints of the residual y - y_obs with the loss 0.5 * ||y - y_obs||^2.
int loss_grad_impl(const EffPlan* plan, const float* x, const float* f, const float* y_obs,
                   double* loss, float* gx, float* gf, char* ws, int batch, void* stream) {
  if (!x || !f || !y_obs) return fail(EFF_ERR_INVALID, "null argument");
  if (!gx && !gf) return fail(EFF_ERR_INVALID, "eff_loss_grad needs gx or gf");
  const Workspace w = workspace_layout(plan, batch);
  float2* xhat = reinterpret_cast<float2*>(ws + w.xhat);
  float2* fhat = reinterpret_cast<float2*>(ws + w.fhat);
  float* y = reinterpret_cast<float*>(ws + w.y);
  // The fused forward accumulates EFF(x, f) - y_obs (each CTA also
  // subtracts its share of the observation, prefetched into L2 at its
  // start), so the adjoint reads one plane, the residual, and takes the loss
  // from it.
  eff::Params P = base_params(plan);
  P.x = x;
  P.f = f;
  P.out0 = y;
  P.out0_bs = P.y_bs;
  P.a_out = gf ? xhat : nullptr;
  P.b_out = gx ? fhat : nullptr;
  P.pf = reinterpret_cast<const char*>(y_obs);
  P.pf_bytes = (long long)sizeof(float) * P.y_bs;
  P.sub = y_obs;
  // the forward also zeroes the adjoint's accumulators (no memset nodes)
  P.zero_f = gx;
  P.zero_nf = gx ? P.x_bs * batch : 0;
  P.zero_d = loss;
  P.zero_nd = loss ? batch : 0;
  if (int s = clear_before(plan, P, y, sizeof(float) * P.y_bs * batch, nullptr, 0, static_cast<cudaStream_t>(stream)))
    return s;
  int s = run(plan, eff::OP_FWD_BOTH, P, batch, stream);
  if (s != EFF_OK) return s;
  // the adjoint may be scheduled while the forward runs (it waits for it)
  return adjoint_impl(plan, y, nullptr, gx ? fhat : nullptr, gf ? xhat : nullptr, gx, gf, loss,
                      EFF_ADJ_EXACT, batch, stream, nullptr, true, true, true);
}

}  // namespace

int eff::set_error(int code, const std::string& msg) { return fail(code, msg); }

int eff::plan_params(const EffPlan* plan, eff::Params* P, int* N) {
  if (!plan) return fail(EFF_ERR_INVALID, "null plan");
  *P = base_params(plan);
  *N = plan->N;
  return EFF_OK;
}

int eff::plan_patches(const EffPlan* plan) { return plan ? plan->K : 0; }

int eff::plan_device(const EffPlan* plan) { return plan ? plan->device : -1; }

bool eff::plan_deterministic(const EffPlan* plan) { return plan && plan->det; }

int eff::check_plan_device(const EffPlan* plan) {
  if (!plan) return fail(EFF_ERR_INVALID, "null plan");
  return check_device(plan);
}

extern "C" {

const char* eff_last_error(void) { return g_last_error.c_str(); }

int eff_plan_create(const EffGeom* geom, const float* win0, const float* win1, EffPlan** plan) {
  if (!geom || !win0 || !win1 || !plan) return fail(EFF_ERR_INVALID, "null argument");
  *plan = nullptr;
  const EffGeom& g = *geom;
  for (int d = 0; d < 2; ++d) {
    if (g.sx[d] < 1 || g.sf[d] < 1 || g.csf[d] < 1 || g.sw[d] < 1 || g.hop[d] < 1)
      return fail(EFF_ERR_INVALID, "sizes must be positive");
    if (g.sf[d] >= g.sx[d])
      return fail(EFF_ERR_INVALID, "Size missmatch: PSF must be smaller than the image");
  }
  if (g.mode < EFF_MODE_VALID || g.mode > EFF_MODE_FULL) return fail(EFF_ERR_INVALID, "Not a valid mode!");
  if (g.flags & ~EFF_GEOM_DETERMINISTIC) return fail(EFF_ERR_INVALID, "unknown geometry flags");
  if ((long long)g.csf[0] * g.csf[1] > 65535) return fail(EFF_ERR_UNSUPPORTED, "too many patches");

  EffPlan p;
  std::memset(&p, 0, sizeof(p));
  p.g = g;
  p.K = g.csf[0] * g.csf[1];
  p.det = (g.flags & EFF_GEOM_DETERMINISTIC) != 0;
  for (int d = 0; d < 2; ++d) {
    p.E[d] = g.sw[d] + g.sf[d] - 1;
    if (g.mode == EFF_MODE_VALID) { p.sy[d] = g.sx[d] - g.sf[d] + 1; p.off[d] = g.sf[d] - 1; }
    else if (g.mode == EFF_MODE_SAME) { p.sy[d] = g.sx[d]; p.off[d] = g.sf[d] / 2; }
    else { p.sy[d] = g.sx[d] + g.sf[d] - 1; p.off[d] = 0; }
  }
  const int emax = p.E[0] > p.E[1] ? p.E[0] : p.E[1];
  if (g.sfft == 0) {
    p.N = 0;
    for (int n : kFrames)
      if (n >= emax) {
        p.N = n;
        break;
      }
    if (p.N == 0) p.N = 1024;  // rejected below
  } else {
    p.N = g.sfft;
  }
  if (!frame_ok(p.N))
    return fail(EFF_ERR_UNSUPPORTED, "FFT frame " + std::to_string(p.N) +
                                         " (needs 64, 128, 192, 256 or 512, >= sw + sf - 1 = " +
                                         std::to_string(emax) + ")");
  if (p.N < emax) return fail(EFF_ERR_INVALID, "FFT frame smaller than sw + sf - 1");
  if (g.threads != 0 && (g.threads < 32 || g.threads % 32 != 0 || g.threads > eff::max_threads(p.N)))
    return fail(EFF_ERR_INVALID, "threads must be 0 or a multiple of 32 in [32, " +
                                     std::to_string(eff::max_threads(p.N)) + "]");

  // Threads per CTA: the most the kernels are compiled for, halved while the
  // frame plus the per-group exchange scratch would not fit in shared memory.
  p.threads = g.threads ? g.threads : eff::max_threads(p.N);
  {
    eff::Params P = base_params(&p);
    P.out0 = reinterpret_cast<float*>(1);
    P.out1 = reinterpret_cast<float*>(1);
    for (;;) {
      size_t worst = 0;
      for (int op = 0; op < eff::kNumOps; ++op) {
        const size_t s = eff::smem_bytes(p.N, op, P, p.threads, 1);
        if (s > worst) worst = s;
      }
      if (worst <= kSmemLimit || p.threads <= 128) break;
      p.threads = (p.threads / 2 + 31) / 32 * 32;
    }
    // 2-CTA clusters: one lane group per column unit a CTA owns (N/4 units
    // of G = N/R lanes) plus a warp in which the DC unit runs alone, at most
    // the compiled maximum, halved while the frame half plus the exchange
    // scratch does not fit.
    p.threads2 = g.threads ? g.threads
                           : std::min(eff::max_threads(p.N),
                                      std::max(128, p.N / 4 * (p.N / eff::lane_values(p.N)) + 32));
    for (;;) {
      size_t worst = 0;
      for (int op = 0; op < eff::kNumOps; ++op) {
        const size_t s = eff::smem_bytes(p.N, op, P, p.threads2, 2);
        if (s > worst) worst = s;
      }
      if (worst <= kSmemLimit || p.threads2 <= 128) break;
      p.threads2 = (p.threads2 / 2 + 31) / 32 * 32;
    }
    // Frame 512 runs on clusters of 4 CTAs (each a quarter of the half
    // spectrum) when a quarter frame fits at the full CTA size, else of 8
    // (fewer rounds per phase than a 4-CTA cluster of smaller CTAs, for the
    // same SM time per patch); the 8-CTA size is halved while it does not fit.
    if (p.N == 512) {
      p.clw = 0;
      for (int cl : {4, 8}) {
        int t = g.threads ? g.threads : eff::max_threads(p.N);
        size_t worst = 0;
        for (;;) {
          worst = 0;
          for (int op = 0; op < eff::kNumOps; ++op) {
            const size_t s = eff::smem_bytes(p.N, op, P, t, cl);
            if (s > worst) worst = s;
          }
          if (worst <= kSmemLimit || cl == 4 || t <= 64) break;
          t = (t / 2 + 31) / 32 * 32;
        }
        if (worst <= kSmemLimit) {
          p.clw = cl;
          p.threads2 = t;
          break;
        }
      }
      if (p.clw == 0)
        return fail(EFF_ERR_UNSUPPORTED, "frame 512: the frame rows (sw + sf - 1 = " + std::to_string(emax) +
                                             ") do not fit in shared memory even split over 8 CTAs");
    }
  }

  cudaError_t e = cudaGetDevice(&p.device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  e = cudaDeviceGetAttribute(&p.num_sms, cudaDevAttrMultiProcessorCount, p.device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");

  // Twiddle table [k1*G + g] = exp(-2 pi i g k1 / N), FP64 then rounded.
  const int R = eff::lane_values(p.N), G = p.N / R;
  std::vector<float2> tw(p.N);
  for (int k1 = 0; k1 < R; ++k1)
    for (int gg = 0; gg < G; ++gg) {
      const double a = -2.0 * M_PI * double(gg * k1) / double(p.N);
      tw[k1 * G + gg] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
  // |FFT([-1, 1])|^2 on N points = 4 sin^2(pi k / N), FP64 then rounded
  // (the Laplacian term of deconv 'xdirect', olaGPU.py:553-561).
  std::vector<float> lap(p.N);
  for (int k = 0; k < p.N; ++k) {
    const double s = std::sin(M_PI * double(k) / double(p.N));
    lap[k] = (float)(4.0 * s * s);
  }
  const size_t n0 = 2 * (size_t)g.csf[0] * g.sw[0], n1 = 2 * (size_t)g.csf[1] * g.sw[1];
  if ((e = cudaMalloc(&p.tw, (sizeof(float2) + sizeof(float)) * p.N + sizeof(int))) != cudaSuccess)
    return cuda_fail(e, "cudaMalloc");
  p.lap = reinterpret_cast<float*>(p.tw + p.N);
  p.err = reinterpret_cast<int*>(p.lap + p.N);
  if ((e = cudaMemset(p.err, 0, sizeof(int))) != cudaSuccess) {
    cudaFree(p.tw);
    return cuda_fail(e, "cudaMemset");
  }
  if ((e = cudaMalloc(&p.win0, sizeof(float) * n0)) != cudaSuccess) {
    cudaFree(p.tw);
    return cuda_fail(e, "cudaMalloc");
  }
  if ((e = cudaMalloc(&p.win1, sizeof(float) * n1)) != cudaSuccess) {
    cudaFree(p.tw);
    cudaFree(p.win0);
    return cuda_fail(e, "cudaMalloc");
  }
  if ((e = cudaMemcpy(p.tw, tw.data(), sizeof(float2) * p.N, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(p.lap, lap.data(), sizeof(float) * p.N, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(p.win0, win0, sizeof(float) * n0, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(p.win1, win1, sizeof(float) * n1, cudaMemcpyHostToDevice)) != cudaSuccess) {
    cudaFree(p.tw);
    cudaFree(p.win0);
    cudaFree(p.win1);
    return cuda_fail(e, "cudaMemcpy");
  }
  if (p.det) {
    const size_t tile = std::max((size_t)p.E[0] * p.E[1], (size_t)g.sw[0] * g.sw[1]);
    if ((e = cudaMalloc(&p.tiles, sizeof(float) * p.K * tile)) != cudaSuccess ||
        (e = cudaMalloc(&p.loss_part, sizeof(double) * p.K * 8)) != cudaSuccess) {
      cudaFree(p.tiles);
      cudaFree(p.tw);
      cudaFree(p.win0);
      cudaFree(p.win1);
      return cuda_fail(e, "cudaMalloc");
    }
  }
  EffPlan* out = new (std::nothrow) EffPlan(p);
  if (!out) {
    cudaFree(p.tiles);
    cudaFree(p.loss_part);
    cudaFree(p.tw);
    cudaFree(p.win0);
    cudaFree(p.win1);
    return fail(EFF_ERR_INVALID, "out of host memory");
  }
  *plan = out;
  return EFF_OK;
}

int eff_plan_destroy(EffPlan* plan) {
  if (!plan) return EFF_OK;
  cudaFree(plan->tw);
  cudaFree(plan->win0);
  cudaFree(plan->win1);
  cudaFree(plan->tiles);
  cudaFree(plan->loss_part);
  delete plan;
  return EFF_OK;
}

int eff_plan_frame(const EffPlan* plan, int* n) {
  if (!plan || !n) return fail(EFF_ERR_INVALID, "null argument");
  *n = plan->N;
  return EFF_OK;
}

size_t eff_spectrum_bytes(const EffPlan* plan) {
  if (!plan) return 0;
  return sizeof(float2) * (size_t)plan->K * (plan->N / 2 + 1) * plan->N;
}

int eff_psf_spectrum(const EffPlan* plan, const float* f, void* fhat, int batch, void* stream) {
  if (int s = check_plan(plan, batch)) return s;
  if (!f || !fhat) return fail(EFF_ERR_INVALID, "null argument");
  eff::Params P = base_params(plan);
  P.f = f;
  P.a_out = static_cast<float2*>(fhat);
  return run(plan, eff::OP_SPEC_PSF, P, batch, stream);
}

int eff_image_spectrum(const EffPlan* plan, const float* x, void* xhat, int batch, void* stream) {
  if (int s = check_plan(plan, batch)) return s;
  if (!x || !xhat) return fail(EFF_ERR_INVALID, "null argument");
  eff::Params P = base_params(plan);
  P.x = x;
  P.a_out = static_cast<float2*>(xhat);
  return run(plan, eff::OP_SPEC_IMAGE, P, batch, stream);
}

int eff_forward_image(const EffPlan* plan, const float* x, const void* fhat, float* y,
                      void* xhat_out, int batch, void* stream) {
  if (int s = check_plan(plan, batch)) return s;
  if (!x || !fhat || !y) return fail(EFF_ERR_INVALID, "null argument");
  eff::Params P = base_params(plan);
  P.x = x;
  P.b0 = static_cast<const float2*>(fhat);
  P.out0 = y;
  P.out0_bs = P.y_bs;
  P.a_out = static_cast<float2*>(xhat_out);
  if (int s = clear_before(plan, P, y, sizeof(float) * P.y_bs * batch, nullptr, 0, static_cast<cudaStream_t>(stream)))
    return s;
  return run(plan, eff::OP_FWD_IMAGE, P, batch, stream);
}

int eff_forward_psf(const EffPlan* plan, const float* f, const void* xhat, float* y,
                    void* fhat_out, int batch, void* stream) {
  if (int s = check_plan(plan, batch)) return s;
  if (!f || !xhat || !y) return fail(EFF_ERR_INVALID, "null argument");
  eff::Params P = base_params(plan);
  P.f = f;
  P.b0 = static_cast<const float2*>(xhat);
  P.out0 = y;
  P.out0_bs = P.y_bs;
  P.a_out = static_cast<float2*>(fhat_out);
  if (int s = clear_before(plan, P, y, sizeof(float) * P.y_bs * batch, nullptr, 0, static_cast<cudaStream_t>(stream)))
    return s;
  return run(plan, eff::OP_FWD_PSF, P, batch, stream);
}

int eff_forward_ex(const EffPlan* plan, int operand, const float* u, const void* spec, float* y, const float* sub,
                   void* spec_out, int flags, float* zero_f, long long zero_nf, double* zero_d, int zero_nd,
                   int batch, void* stream) {
  if (int s = check_plan(plan, batch)) return s;
  if (!u || !spec || !y) return fail(EFF_ERR_INVALID, "null argument");
  if (sub == y) return fail(EFF_ERR_INVALID, "sub must not alias y");
  if (operand != EFF_OPERAND_IMAGE && operand != EFF_OPERAND_PSF) return fail(EFF_ERR_INVALID, "operand");
  if ((flags & ~EFF_OUT_ZEROED) || zero_nf < 0 || zero_nd < 0 || (zero_nf > 0 && !zero_f) || (zero_nd > 0 && !zero_d))
    return fail(EFF_ERR_INVALID, "bad argument");
  eff::Params P = base_params(plan);
  if (operand == EFF_OPERAND_IMAGE) P.x = u;
  else P.f = u;
  P.b0 = static_cast<const float2*>(spec);
  P.out0 = y;
  P.out0_bs = P.y_bs;
  P.sub = sub;
  P.a_out = static_cast<float2*>(spec_out);
  P.zero_f = zero_nf > 0 ? zero_f : nullptr;
  P.zero_nf = zero_nf;
  P.zero_d = zero_nd > 0 ? zero_d : nullptr;
  P.zero_nd = zero_nd;
  if (!(flags & EFF_OUT_ZEROED)) {
    if (int s = clear_before(plan, P, y, sizeof(float) * P.y_bs * batch, nullptr, 0, static_cast<cudaStream_t>(stream)))
      return s;
  }
  return run(plan, operand == EFF_OPERAND_IMAGE ? eff::OP_FWD_IMAGE : eff::OP_FWD_PSF, P, batch, stream);
}

int eff_adjoint_ex(const EffPlan* plan, const float* y, const float* y_obs, const float* mask, const void* fhat,
                   const void* xhat, float* gx, float* gf, double* loss, int adj_mode, int flags, int batch,
                   void* stream) {
  if (flags & ~(EFF_OUT_ZEROED | EFF_LOSS_OF_Y | EFF_AFTER_FORWARD)) return fail(EFF_ERR_INVALID, "flags");
  const bool loss_y = (flags & EFF_LOSS_OF_Y) != 0;
  if (loss_y && (y_obs || mask)) return fail(EFF_ERR_INVALID, "EFF_LOSS_OF_Y takes no y_obs or mask");
  if (loss && !y_obs && !loss_y) return fail(EFF_ERR_INVALID, "the loss needs y_obs (or EFF_LOSS_OF_Y)");
  return adjoint_impl(plan, y, y_obs, fhat, xhat, gx, gf, loss, adj_mode, batch, stream, mask,
                      (flags & EFF_OUT_ZEROED) != 0, loss_y, (flags & EFF_AFTER_FORWARD) != 0);
}

int eff_adjoint(const EffPlan* plan, const float* y, const void* fhat, const void* xhat, float* gx,
                float* gf, int adj_mode, int batch, void* stream) {
  return adjoint_impl(plan, y, nullptr, fhat, xhat, gx, gf, nullptr, adj_mode, batch, stream);
}

int eff_adjoint_residual(const EffPlan* plan, const float* y, const float* y_obs, const void* fhat,
                         const void* xhat, float* gx, float* gf, double* loss, int adj_mode,
                         int batch, void* stream) {
  if (!y_obs) return fail(EFF_ERR_INVALID, "null y_obs");
  return adjoint_impl(plan, y, y_obs, fhat, xhat, gx, gf, loss, adj_mode, batch, stream);
}

int eff_deconv_xdirect(const EffPlan* plan, const float* y, const void* fhat, const void* xhat, float* u,
                       float* fz, float alpha, float beta, int batch, void* stream) {
  if (int s = check_plan(plan, batch)) return s;
  if (!y || (!u && !fz)) return fail(EFF_ERR_INVALID, "null argument");
  if (u && !fhat) return fail(EFF_ERR_INVALID, "image estimate needs the PSF spectrum");
  if (fz && !xhat) return fail(EFF_ERR_INVALID, "PSF estimate needs the image spectrum");
  if (plan->g.mode == EFF_MODE_FULL) return fail(EFF_ERR_UNSUPPORTED, "Not a valid mode!");  // olaGPU.py:570-571
  if (!(alpha >= 0.f) || !(beta >= 0.f)) return fail(EFF_ERR_INVALID, "alpha and beta must be >= 0");
  eff::Params P = base_params(plan);
  P.y = y;
  P.b0 = static_cast<const float2*>(fhat);
  P.b1 = static_cast<const float2*>(xhat);
  P.out0 = u;
  P.out1 = fz;
  P.out0_bs = P.x_bs;
  P.out1_bs = P.f_bs;
  // the chop of y sits at frame offset `off` (sf - 1 valid, floor(sf/2) same)
  P.lo0 = plan->off[0];
  P.lo1 = plan->off[1];
  P.alpha = alpha;
  P.beta = beta;
  if (int s = clear_before(plan, P, u, sizeof(float) * P.x_bs * batch, nullptr, 0, static_cast<cudaStream_t>(stream)))
    return s;
  return run(plan, eff::OP_DECONV, P, batch, stream);
}

int eff_adjoint_masked(const EffPlan* plan, const float* y, const float* mask, const void* fhat,
                       const void* xhat, float* gx, float* gf, int adj_mode, int batch, void* stream) {
  if (!mask) return fail(EFF_ERR_INVALID, "null mask");
  return adjoint_impl(plan, y, nullptr, fhat, xhat, gx, gf, nullptr, adj_mode, batch, stream, mask);
}

int eff_forward_both(const EffPlan* plan, const float* x, const float* f, float* y, void* xhat_out,
                     void* fhat_out, int batch, void* stream) {
  if (int s = check_plan(plan, batch)) return s;
  if (!x || !f || !y) return fail(EFF_ERR_INVALID, "null argument");
  eff::Params P = base_params(plan);
  P.x = x;
  P.f = f;
  P.out0 = y;
  P.out0_bs = P.y_bs;
  P.a_out = static_cast<float2*>(xhat_out);
  P.b_out = static_cast<float2*>(fhat_out);
  if (int s = clear_before(plan, P, y, sizeof(float) * P.y_bs * batch, nullptr, 0, static_cast<cudaStream_t>(stream)))
    return s;
  return run(plan, eff::OP_FWD_BOTH, P, batch, stream);
}

int eff_forward_residual(const EffPlan* plan, const float* x, const float* f, const float* y_obs, float* r,
                         void* xhat_out, void* fhat_out, int batch, void* stream) {
  if (int s = check_plan(plan, batch)) return s;
  if (!x || !f || !y_obs || !r) return fail(EFF_ERR_INVALID, "null argument");
  if (r == y_obs) return fail(EFF_ERR_INVALID, "r must not alias y_obs");
  eff::Params P = base_params(plan);
  P.x = x;
  P.f = f;
  P.out0 = r;
  P.out0_bs = P.y_bs;
  P.a_out = static_cast<float2*>(xhat_out);
  P.b_out = static_cast<float2*>(fhat_out);
  P.pf = reinterpret_cast<const char*>(y_obs);
  P.pf_bytes = (long long)sizeof(float) * P.y_bs;
  P.sub = y_obs;
  if (int s = clear_before(plan, P, r, sizeof(float) * P.y_bs * batch, nullptr, 0, static_cast<cudaStream_t>(stream)))
    return s;
  return run(plan, eff::OP_FWD_BOTH, P, batch, stream);
}

int eff_forward_both_ex(const EffPlan* plan, const float* x, const float* f, const float* sub, float* y,
                        void* xhat_out, void* fhat_out, int flags, float* zero_f, long long zero_nf, double* zero_d,
                        int zero_nd, int batch, void* stream) {
  if (int s = check_plan(plan, batch)) return s;
  if (!x || !f || !y) return fail(EFF_ERR_INVALID, "null argument");
  if (sub == y) return fail(EFF_ERR_INVALID, "sub must not alias y");
  if ((flags & ~EFF_OUT_ZEROED) || zero_nf < 0 || zero_nd < 0 || (zero_nf > 0 && !zero_f) || (zero_nd > 0 && !zero_d))
    return fail(EFF_ERR_INVALID, "bad argument");
  eff::Params P = base_params(plan);
  P.x = x;
  P.f = f;
  P.out0 = y;
  P.out0_bs = P.y_bs;
  P.a_out = static_cast<float2*>(xhat_out);
  P.b_out = static_cast<float2*>(fhat_out);
  if (sub) {
    P.pf = reinterpret_cast<const char*>(sub);
    P.pf_bytes = (long long)sizeof(float) * P.y_bs;
    P.sub = sub;
  }
  P.zero_f = zero_nf > 0 ? zero_f : nullptr;
  P.zero_nf = zero_nf;
  P.zero_d = zero_nd > 0 ? zero_d : nullptr;
  P.zero_nd = zero_nd;
  if (!(flags & EFF_OUT_ZEROED)) {
    if (int s = clear_before(plan, P, y, sizeof(float) * P.y_bs * batch, nullptr, 0, static_cast<cudaStream_t>(stream)))
      return s;
  }
  return run(plan, eff::OP_FWD_BOTH, P, batch, stream);
}

size_t eff_loss_grad_workspace_bytes(const EffPlan* plan, int batch) {
  if (!plan || batch < 1) return 0;
  return workspace_layout(plan, batch).total;
}

int eff_loss_grad(const EffPlan* plan, const float* x, const float* f, const float* y_obs,
                  double* loss, float* gx, float* gf, void* workspace, size_t workspace_bytes,
                  int batch, void* stream) {
  if (int s = check_plan(plan, batch)) return s;
  if (!workspace) return fail(EFF_ERR_INVALID, "null workspace");
  const Workspace w = workspace_layout(plan, batch);
  if (workspace_bytes < w.total)
    return fail(EFF_ERR_INVALID, "workspace too small: need " + std::to_string(w.total) + " bytes");
  return loss_grad_impl(plan, x, f, y_obs, loss, gx, gf, static_cast<char*>(workspace), batch, stream);
}

int eff_project_psf(float* f, int K, int n, int proj_mode, void* stream) {
  if (!f || K < 1 || n < 1) return fail(EFF_ERR_INVALID, "bad argument");
  if (proj_mode != EFF_PROJ_CLIP_NORMALIZE && proj_mode != EFF_PROJ_SIMPLEX)
    return fail(EFF_ERR_INVALID, "proj_mode");
  cudaError_t e = eff::launch_project(f, K, n, proj_mode, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "projection launch");
  return EFF_OK;
}

int eff_basis_project(const float* fs, const float* basis, float* w, int nb, int n, void* stream) {
  if (!fs || !basis || !w || nb < 1 || n < 1) return fail(EFF_ERR_INVALID, "bad argument");
  cudaError_t e = eff::launch_basis_project(fs, basis, w, nb, n, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "basis projection launch");
  return EFF_OK;
}

int eff_edgetaper(float* im, int rows, int cols, const float* wy, int hy, const float* wx, int hx,
                  int batch, void* stream) {
  if (!im || rows < 1 || cols < 1 || batch < 1 || batch > 65535 || hy < 0 || hx < 0 ||
      (hy > 0 && !wy) || (hx > 0 && !wx) || 2 * hy > rows || 2 * hx > cols)
    return fail(EFF_ERR_INVALID, "bad argument");
  cudaError_t e = eff::launch_edgetaper(im, rows, cols, wy, hy, wx, hx, batch, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "edgetaper launch");
  return EFF_OK;
}

int eff_dots3(const float* a, const float* ap, long long na, const float* b, const float* bp, long long nb,
              double* out, int flags, void* stream) {
  if (!a || !b || !out || na < 1 || nb < 1 || (flags & ~EFF_OUT_ZEROED)) return fail(EFF_ERR_INVALID, "bad argument");
  cudaError_t e = eff::launch_dots3(a, ap, na, b, bp, nb, out, (flags & EFF_OUT_ZEROED) != 0,
                                    static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "dots3 launch");
  return EFF_OK;
}

int eff_pg_step(float* f, const float* g, float* f_prev, float* g_prev, int K, int n, const double* dots,
                int mode, float* state, float* zero_f, long long zero_n, void* stream) {
  if (!f || !g || !f_prev || !g_prev || !dots || !state || K < 1 || n < 1 || mode < 0 || mode > 2 ||
      zero_n < 0 || (zero_n > 0 && !zero_f))
    return fail(EFF_ERR_INVALID, "bad argument");
  if (n > 12288) return fail(EFF_ERR_UNSUPPORTED, "PSF larger than 12288 samples");
  cudaError_t e = eff::launch_pg_step(f, g, f_prev, g_prev, K, n, dots, mode, state, zero_f, zero_n,
                                      static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "pg_step launch");
  return EFF_OK;
}

int eff_max_nonneg(const float* a, long long n, unsigned* out_bits, void* stream) {
  if (!a || !out_bits || n < 1) return fail(EFF_ERR_INVALID, "bad argument");
  cudaError_t e = eff::launch_max_nonneg(a, n, out_bits, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "max launch");
  return EFF_OK;
}

int eff_mu_update(float* x, const float* num, const float* den, float tol, int rows, int cols, int border0,
                  int border1, const unsigned* num_max_bits, float floor_rel, unsigned* xmax_bits, int flags,
                  float* zero_f, long long zero_n, void* stream) {
  if (!x || !num || !den || !xmax_bits || !num_max_bits || rows < 1 || cols < 1 || border0 < 0 ||
      border1 < 0 || !(floor_rel >= 0.f) || (flags & ~EFF_OUT_ZEROED) || zero_n < 0 || (zero_n > 0 && !zero_f))
    return fail(EFF_ERR_INVALID, "bad argument");
  cudaError_t e = eff::launch_mu_update(x, num, den, tol, rows, cols, border0, border1, num_max_bits,
                                        floor_rel, xmax_bits, (flags & EFF_OUT_ZEROED) != 0, zero_f, zero_n,
                                        static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "mu_update launch");
  return EFF_OK;
}

int eff_plan_device_errors(const EffPlan* plan, int* flags, int clear) {
  if (!plan || !flags) return fail(EFF_ERR_INVALID, "null argument");
  if (int s = check_device(plan)) return s;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(flags, plan->err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && clear) e = cudaMemset(plan->err, 0, sizeof(int));
  if (e != cudaSuccess) return cuda_fail(e, "reading the device error word");
  return EFF_OK;
}

int eff_set_image_tile(int on) {
  if (on != 0 && on != 1) return fail(EFF_ERR_INVALID, "image tile must be 0 or 1");
  g_image_tile.store(on);
  return EFF_OK;
}

int eff_set_spectrum_staging(int on) {
  if (on < 0 || on > 2) return fail(EFF_ERR_INVALID, "spectrum staging must be 0, 1 or 2");
  g_stage_spectra.store(on);
  return EFF_OK;
}

int eff_test_plan_set_device(EffPlan* plan, int device) {
  if (!plan) return fail(EFF_ERR_INVALID, "null plan");
  plan->device = device;
  return EFF_OK;
}

int eff_set_cluster_mode(int mode) {
  if (mode < 0 || mode > 2) return fail(EFF_ERR_INVALID, "cluster mode must be 0, 1 or 2");
  g_cluster_mode.store(mode);
  return EFF_OK;
}

}  // extern "C"
