// Fused EFF kernels: one CTA per patch (blockIdx.x) and image (blockIdx.y).
//
// Every kernel runs the same three phases over an N x N frame (N = 64, 128,
// 192 or 256, >= sw + sf - 1 in both dims) held as a half spectrum
// (N/2+1 bins per row) in shared memory:
//
//  1. row pass (R2C): pairs of real operand rows are read straight from HBM
//     (windowed image patch, PSF, or the output-side image / residual for the
//     adjoints), packed as one complex row, transformed, and split into two
//     half-spectrum rows.  Kernels with two operands run both in one loop.
//  2. column pass: each lane group takes one column (columns 0 and N/2, both
//     real after the row pass, share one complex transform), transforms it,
//     optionally stores it as a cached spectrum, multiplies it by the other
//     operand's spectrum (conjugated for the adjoints) and inverse transforms
//     it, all in registers; only the rows the epilogue needs go back to
//     shared memory.
//  3. row pass (C2R): pairs of half-spectrum rows are inverse transformed as
//     one complex row; the epilogue overlap-adds into the output image with
//     fp32 atomics (forward: full-convolution extent, cropped by mode; image
//     adjoint: windowed, patch extent) or stores the PSF gradient.
//
// With CL = 2 a patch is processed by a cluster of two CTAs: CTA c owns the
// column units [c*N/4, (c+1)*N/4) of the half spectrum (CTA 0 also the N/2
// bin) in its shared memory; the row passes write and read the peer's
// columns through distributed shared memory, the column pass is local.
//
// Reference semantics: OlaGPU.cnv / OlaGPU.cnvtp, olaGPU.py:170-311.
#pragma once
#include <cooperative_groups.h>
#include <cuda.h>  // CUtensorMap (the type only; maps are encoded on the host)

#include "eff_fft.cuh"

namespace eff {
namespace cg = cooperative_groups;

enum Op : int {
  OP_SPEC_IMAGE = 0,  // X-hat of the windowed patches (OlaGPU X object, olaGPU.py:147-157)
  OP_SPEC_PSF = 1,    // F-hat of the PSFs (OlaGPU F object, olaGPU.py:142-157)
  OP_FWD_IMAGE = 2,   // y = F x, F given by F-hat (F.cnv(x), olaGPU.py:200-257)
  OP_FWD_PSF = 3,     // y = X f, X given by X-hat (X.cnv(f), olaGPU.py:188-193, 219-257)
  OP_FWD_BOTH = 4,    // y = EFF(x, f) from raw x and f; leaves X-hat and F-hat behind
  OP_ADJ = 5,         // F^T r and/or X^T r (cnvtp, olaGPU.py:261-311), r = y or y - y_obs
  OP_DECONV = 6,      // Fourier-division deconvolution of y (deconv 'xdirect', olaGPU.py:550-609)
};
constexpr int kNumOps = 7;

enum Operand : int { OPND_IMAGE = 0, OPND_PSF = 1, OPND_RESID = 2, OPND_DCHOP = 3 };

struct Params {
  int sx0, sx1, sf0, sf1, csf0, csf1, sw0, sw1, hop0, hop1;
  int sy0, sy1, off0, off1, E0, E1;
  int lo0, hi0, lo1, hi1;  // adjoint input window inside a frame
  const float* x;          // image [sx0, sx1]
  const float* f;          // PSFs [K, sf0, sf1]
  const float* y;          // output-side image [sy0, sy1] (adjoint input)
  const float* y_obs;      // adjoint: when set, the input is y - y_obs
  const float* mask;       // adjoint: when set, the input is multiplied by mask [sy0, sy1]
  const float2* b0;        // cached spectrum: F-hat (fwd image / adj image) or X-hat (fwd psf)
  const float2* b1;        // cached spectrum: X-hat (adj psf)
  float2* a_out;           // spectrum of operand A (optional)
  float2* b_out;           // spectrum of operand B (OP_FWD_BOTH, optional)
  float* out0;             // y (forward) or gx (image adjoint)
  float* out1;             // gf (PSF adjoint)
  double* loss;            // adjoint with y_obs: += 0.5 * sum (y - y_obs)^2 (optional)
  const float2* win0;      // window factors (alpha, gamma) [csf0, sw0]
  const float2* win1;      // window factors (alpha, gamma) [csf1, sw1]
  const float2* tw;        // W_N table [R*G] = [N]
  long long x_bs, f_bs, y_bs, spec_bs, out0_bs, out1_bs;  // per-image strides
  const char* pf;          // forward: bytes [pf, pf + pf_bytes) to bring into L2 for the next kernel
  long long pf_bytes;
  const float* lap;        // deconv: 4 sin^2(pi k / N), k < N (spectrum of the difference filters)
  float alpha, beta;       // deconv: regularisation weights
  float* zero_f;           // eff_kernel: zero [zero_f, zero_f + zero_nf) (the next kernel's
  long long zero_nf;       //   accumulator), spread over the grid
  double* zero_d;          // eff_kernel: zero [zero_d, zero_d + zero_nd)
  int zero_nd;
  const float* sub;        // forward: subtract this plane [sy0, sy1] from out0 too (a share per CTA, by
                           //   atomics), so that out0 ends as EFF(...) - sub
  int loss_y;              // adjoint without y_obs: loss += 0.5 * sum y^2 (y is already the residual)
  int stage_spec;          // eff_kernel: copy this CTA's columns of the cached spectra into shared
                           //   memory (cp.async.bulk) at kernel start (host: only where they fit)
  int* err;                // device error word of the plan (bit 0: a bulk copy did not complete in time)
  float* tiles;            // deterministic overlap-add: the forward stores patch k's E0 x E1 output tile
                           //   (the image adjoint / deconvolution its sw0 x sw1 tile) at
                           //   tiles + (b K + k) * tile size, instead of adding it into the image;
                           //   ola_gather sums the tiles in a fixed order
  double* loss_part;       // deterministic loss: each CTA stores its share at loss_part[b ncta + cta]
  int tile_rows, tile_w;   // image operand by the tensor engine (tile_rows > 0, kernels given a
                           //   tensor map of x): a tile_rows x tile_w box of the patch's window
                           //   per CTA into shared memory at kernel start (zero outside the image)
  int pdl;                 // launched with programmatic stream serialization: 1 = right after
                           //   the kernel whose results it reads, wait (griddepcontrol.wait)
                           //   first; 2 = right after the zero kernel clearing its accumulated
                           //   outputs, wait before the output phase
};

// TMA bulk prefetch of a contiguous range into L2 (16-byte aligned start and
// size, sm_90+).
__device__ __forceinline__ void l2_prefetch_bulk(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// --- bulk copies into shared memory, completed on an mbarrier -------------
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
// Contiguous global -> this CTA's shared memory (16-byte aligned, size a
// multiple of 16), counted on bar.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
// Box at (c0, c1, c2) of a rank-3 tensor map -> this CTA's shared memory
// (128-byte aligned), counted on bar.  c0 * 4 bytes must be a multiple of 16.
__device__ __forceinline__ void tensor_copy_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2,
                                               unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar))
      : "memory");
}
// Shared-memory address of this CTA's `a` in cluster CTA `rank`.
__device__ __forceinline__ unsigned cluster_addr(unsigned a, unsigned rank) {
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
// Asynchronous store of v to cluster shared-memory address `dst`, counted as
// 8 bytes on the mbarrier at cluster address `bar` (in the destination CTA).
__device__ __forceinline__ void store_async(unsigned dst, float2 v, unsigned bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f32 [%0], {%1, %2}, [%3];" ::"r"(dst),
               "f"(v.x), "f"(v.y), "r"(bar)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Wait for phase `parity` of bar with an iteration limit (each try_wait may
// suspend the thread for a while): false when the limit ran out.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity) {
  for (int i = 0; i < (1 << 22); ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
constexpr int kErrCopyTimeout = 1;
constexpr int kErrBounds = 2;

// Debug builds (-DEFF_DEBUG, the library's checked variant): every frame and
// global index the kernels form is tested against its buffer before the
// access; a bad index sets kErrBounds in the plan's device error word and
// the access is skipped, so the kernel runs to its end and the host can read
// the error.  In the product build EFF_IN is the constant true.
#ifdef EFF_DEBUG
__device__ __forceinline__ bool dbg_in(long long i, long long n, int* err) {
  if (i >= 0 && i < n) return true;
  if (err) atomicOr(err, kErrBounds);
  return false;
}
#define EFF_IN(i, n, err) ::eff::dbg_in((long long)(i), (long long)(n), (err))
#else
#define EFF_IN(i, n, err) true
#endif

// Half-spectrum bins a CTA stores per row: all N/2+1 (CL = 1) or its
// quarter plus, on CTA 0, the N/2 bin (CL = 2).
__host__ __device__ constexpr int frame_pitch(int N, int CL = 1) { return CL == 1 ? N / 2 + 1 : N / (2 * CL) + 1; }
__host__ __device__ constexpr int even_up(int v) { return (v + 1) & ~1; }
// Threads per CTA the kernel is compiled for (the host may launch fewer).
__host__ __device__ constexpr int max_threads(int N) {
  return N % 3 == 0 ? 384 : (N == 256 ? 576 : (N == 128 ? 544 : 512));
}

// Operand A / B of each op, their row counts and frame bases.
__host__ __device__ constexpr int opnd_a(int op) {
  return (op == OP_SPEC_PSF || op == OP_FWD_PSF)
             ? OPND_PSF
             : (op == OP_ADJ ? OPND_RESID : (op == OP_DECONV ? OPND_DCHOP : OPND_IMAGE));
}
__host__ __device__ constexpr bool has_b(int op) { return op == OP_FWD_BOTH; }

__host__ __device__ inline int opnd_rows(const Params& P, int kind) {
  return (kind == OPND_IMAGE || kind == OPND_DCHOP) ? P.sw0 : (kind == OPND_PSF ? P.sf0 : P.E0);
}

// Frame rows a CTA uses (the host sizes shared memory with the same formula).
__host__ __device__ inline int frame_rows(const Params& P, int op) {
  const int ra = even_up(opnd_rows(P, opnd_a(op)));
  if (op == OP_SPEC_IMAGE || op == OP_SPEC_PSF) return ra;
  if (op == OP_FWD_IMAGE || op == OP_FWD_PSF) return max(ra, even_up(P.E0));
  if (op == OP_FWD_BOTH) return max(ra + even_up(P.sf0), even_up(P.E0));
  const int r0 = P.out0 ? even_up(P.sw0) : 0;
  const int r1 = P.out1 ? even_up(P.sf0) : 0;
  return max(ra, r0 + r1);
}

// Cached spectra staged in shared memory: how many (in order b0, b1), the
// columns a CTA keeps of each (its W bins plus a slot for bin N/2, used on
// CTA 0), and the padding per column (spreads the four lane groups of a
// warp, which read four neighbouring columns, over the banks).
constexpr int kSpecPad = 8;
__host__ __device__ inline int staged_specs(const Params& P, int op) {
  if (!P.stage_spec) return 0;
  if (op == OP_FWD_IMAGE || op == OP_FWD_PSF) return 1;
  if (op == OP_ADJ || op == OP_DECONV) return (P.out0 ? 1 : 0) + (P.out1 ? 1 : 0);
  return 0;
}
__host__ __device__ constexpr int staged_cols(int N, int CL) { return N / (2 * CL) + 1; }

// Output rows of the frame-128 pair (2-CTA cluster): the inverse column
// transforms of phase 2 put each frame row into the CTA that runs its
// inverse row transform in phase 3 (CTA c owns row pairs [c U3, (c+1) U3)),
// into a full-width row block there -- the peer's rows by asynchronous
// remote stores that complete on the peer's mbarrier -- so that phase 3
// reads only its own shared memory and waits on that mbarrier instead of a
// cluster barrier.  Forwards and the deconvolution (512^2 step 36.2 -> 35.7
// us, deconvolution 27.4 -> 26.2 us); not the adjoint, whose two outputs
// double the remote stores (+0.6 us).
__host__ __device__ constexpr bool row_owned(int N, int CL, int op) {
  return N == 128 && CL == 2 && op != OP_ADJ;
}
// Row pairs phase 3 transforms.
__host__ __device__ inline int phase3_units(const Params& P, int op) {
  if (op == OP_FWD_IMAGE || op == OP_FWD_PSF || op == OP_FWD_BOTH) return (P.E0 + 1) >> 1;
  if (op == OP_ADJ || op == OP_DECONV) return (P.out0 ? (P.sw0 + 1) >> 1 : 0) + (P.out1 ? (P.sf0 + 1) >> 1 : 0);
  return 0;
}
// Row pairs per CTA of the row-owned output block (0 where it is not used).
__host__ __device__ inline int phase3_pairs(const Params& P, int op, int N, int CL) {
  return row_owned(N, CL, op) ? (phase3_units(P, op) + CL - 1) / CL : 0;
}
__host__ __device__ constexpr int out_pitch(int N) { return N / 2 + 1; }
// Shared memory (float2) of the row-owned block and its mbarrier.
__host__ __device__ inline int out_rows_f2(const Params& P, int op, int N, int CL) {
  const int u3 = phase3_pairs(P, op, N, CL);
  return u3 ? 2 * u3 * out_pitch(N) + 1 : 0;
}
// Shared memory (float2) of the image tile: up to 15 slots to a 128-byte
// boundary, the tile, the mbarrier.
__host__ __device__ inline int image_tile_f2(const Params& P, int op) {
  if (opnd_a(op) != OPND_IMAGE || P.tile_rows <= 0) return 0;
  return 15 + (P.tile_rows * P.tile_w + 1) / 2 + 1;
}

template <int N>
__device__ __forceinline__ unsigned group_mask(int lane) {
  constexpr int G = FftShape<N>::G;
  return G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
}

// The half-spectrum frame of one patch, possibly split over a cluster of CL
// CTAs: CTA c owns the W = N/(2 CL) bins [c W, (c+1) W), CTA 0 also bin N/2
// (at local column W).
template <int N, int CL>
struct Frame {
  static constexpr int HP = frame_pitch(N, CL);
  static constexpr int W = CL == 1 ? N / 2 : N / (2 * CL);
  float2* part[CL];  // generic pointers to every CTA's frame (own one included)
  float2* local;     // this CTA's frame (shared window)
  int rank;
  int rows;          // frame rows of every CTA (bound of the debug build's checks)
  int* err;          // plan's device error word (debug build)
  // Owner and local column of half-spectrum bin b.
  __device__ __forceinline__ static int owner(int b) { return (CL == 1 || b == N / 2) ? 0 : b / W; }
  __device__ __forceinline__ static int lcol(int b) {
    return CL == 1 ? b : (b == N / 2 ? W : b - (b / W) * W);
  }
  __device__ __forceinline__ float2* at(int row, int b) const {
    // CL = 2, frames up to 128: a select, so that the two pointers stay in
    // registers (an index into part[] puts the array in local memory and
    // adds a dependent load to every frame access; the frame-256 kernels
    // have no registers to spare for it: their forward spills more)
    if constexpr (CL == 2 && N <= 128) return (owner(b) ? part[1] : part[0]) + row * HP + lcol(b);
    else return part[owner(b)] + row * HP + lcol(b);
  }
  static constexpr int kDcN = W;  // local column of bin N/2 (CTA 0; the DC unit packs it with column 0)
};

// The row-owned output block (row_owned(N, CL, op), CL = 2): frame row rho
// (pair rho / 2) lives on CTA c = (rho / 2 >= U3) at block row
// rho - 2 c U3, every half-spectrum bin at its own column.
template <int N>
struct OutRows {
  static constexpr int OP3 = out_pitch(N);
  float2* local;  // this CTA's block; its mbarrier follows the block
  int rank, U3;
  int* err;       // plan's device error word (debug build)
};

// One overlap-add contribution: an atomic add into the output image, or, for
// a deterministic plan, a plain store into the patch's tile (every tile
// element is written once).  One predicated pair of instructions, so that the
// epilogues keep a single code path for both.
__device__ __forceinline__ void ola_put(float* p, float v, bool tile) {
  asm volatile(
      "{\n .reg .pred q;\n setp.ne.u32 q, %2, 0;\n @q st.global.f32 [%0], %1;\n @!q red.global.add.f32 [%0], %1;\n}" ::"l"(p),
      "f"(v), "r"((unsigned)tile)
      : "memory");
}

// Window weight ws[k=(m,n)][r][c] from the per-dim (alpha, gamma) tables:
// alpha*alpha' inside the image, gamma*gamma' = 1/(patches covering the
// pixel) on the outermost rows/columns that only zero-valued window samples
// reach (alpha < 0 marks them).  That is the reference's partition of unity
// w / chop(ola(w)) with w floored at 1e-16 (imagetools.py:341, 437-445).
__device__ __forceinline__ float window_weight(float2 u, float2 v) {
  return (u.x < 0.f || v.x < 0.f) ? u.y * v.y : u.x * v.x;
}

struct Patch {
  int m, n, k;
  const float* x;
  const float* f;
  const float* y;
  const float* y_obs;
  const float* mask;
};

// Operand value at frame position (r, c) of the PSF and deconvolution-chop
// operands (the image and residual operands have row loaders of their own).
template <int KIND>
__device__ __forceinline__ float operand(const Params& P, const Patch& T, int r, int c) {
  static_assert(KIND == OPND_PSF || KIND == OPND_DCHOP, "image / residual rows: load_image_rows / load_resid_rows");
  if constexpr (KIND == OPND_PSF) {
    if (r >= P.sf0 || c >= P.sf1) return 0.f;
    const long long q = ((long long)T.k * P.sf0 + r) * P.sf1 + c;
    if (!EFF_IN(q, (long long)P.csf0 * P.csf1 * P.sf0 * P.sf1, P.err)) return 0.f;
    return __ldg(T.f + q);
  } else {
    // deconv 'xdirect': chop of y placed at frame offset lo (chop_pad_GPU,
    // olaGPU.py:573-580) times the window stack at the frame origin
    // (pad_stack_GPU(ws), :581-584); the supports overlap on [lo, sw)
    if (r < P.lo0 || r >= P.sw0 || c < P.lo1 || c >= P.sw1) return 0.f;
    const int i = T.m * P.hop0 + r - P.lo0, j = T.n * P.hop1 + c - P.lo1;
    if (i >= P.sy0 || j >= P.sy1) return 0.f;
    if (!EFF_IN((long long)i * P.sy1 + j, (long long)P.sy0 * P.sy1, P.err) ||
        !EFF_IN(T.m * P.sw0 + r, P.csf0 * P.sw0, P.err) || !EFF_IN(T.n * P.sw1 + c, P.csf1 * P.sw1, P.err))
      return 0.f;
    return window_weight(__ldg(P.win0 + T.m * P.sw0 + r), __ldg(P.win1 + T.n * P.sw1 + c)) *
           __ldg(T.y + (long long)i * P.sy1 + j);
  }
}

// Residual rows (ra, ra+1) of the output-side image: frame position (r, c)
// holds y[i, j] (OBS: minus y_obs[i, j]; MSK: times mask[i, j]) at
// i = m*hop0 + r - off0, j = n*hop1 + c - off1 inside [lo, hi) of the frame
// and inside the image, else 0.  Which rows and which column range
// [clo, chi) hold data is worked out once per row pair, so the loads are a
// straight run of independent reads.
template <int N, bool OBS, bool MSK>
__device__ __forceinline__ void load_resid_rows(const Params& P, const Patch& T, int ra, int g,
                                                float2 (&v)[FftShape<N>::R]) {
  constexpr int G = FftShape<N>::G;
  constexpr int R = FftShape<N>::R;
  const int i0 = T.m * P.hop0 + ra - P.off0;
  const bool okA = ra >= P.lo0 && ra < P.hi0 && i0 >= 0 && i0 < P.sy0;
  const bool okB = ra + 1 >= P.lo0 && ra + 1 < P.hi0 && i0 + 1 >= 0 && i0 + 1 < P.sy0;
  const int jb = T.n * P.hop1 - P.off1;  // frame column c is image column jb + c
  const int clo = max(P.lo1, -jb), chi = min(P.hi1, P.sy1 - jb);
  const long long oa = (long long)i0 * P.sy1 + jb, ob = oa + P.sy1;
#pragma unroll
  for (int mm = 0; mm < R; ++mm) {
    const int c = g + G * mm;
    const bool cv = c >= clo && c < chi && (!okA || EFF_IN(oa + c, (long long)P.sy0 * P.sy1, P.err)) &&
                    (!okB || EFF_IN(ob + c, (long long)P.sy0 * P.sy1, P.err));
    float a = 0.f, b = 0.f;
    if (cv && okA) {
      a = __ldg(T.y + (oa + c));
      if constexpr (OBS) a -= __ldg(T.y_obs + (oa + c));
      if constexpr (MSK) a *= __ldg(T.mask + (oa + c));
    }
    if (cv && okB) {
      b = __ldg(T.y + (ob + c));
      if constexpr (OBS) b -= __ldg(T.y_obs + (ob + c));
      if constexpr (MSK) b *= __ldg(T.mask + (ob + c));
    }
    v[mm] = make_float2(a, b);
  }
}

// Windowed image rows (ra, ra+1): frame position (r, c) holds
// window_weight(win0[m][r], win1[n][c]) * x[m*hop0 + r, n*hop1 + c] for
// r < sw0, c < sw1 inside the image, else 0; the rows' window factors and the
// valid column range are taken once per row pair.
template <int N>
__device__ __forceinline__ void load_image_rows(const Params& P, const Patch& T, int ra, int g,
                                                float2 (&v)[FftShape<N>::R], const float* tile = nullptr,
                                                int t_r0 = 0) {
  constexpr int G = FftShape<N>::G;
  constexpr int R = FftShape<N>::R;
  const int i0 = T.m * P.hop0 + ra;
  // rows of this CTA's image tile (shared memory): the same values, one
  // shared-memory read each
  if (tile && ra >= t_r0 && ra + 1 < t_r0 + P.tile_rows) {
    const bool okA = ra < P.sw0 && i0 < P.sx0;
    const bool okB = ra + 1 < P.sw0 && i0 + 1 < P.sx0;
    const float2 wa = okA ? __ldg(P.win0 + T.m * P.sw0 + ra) : make_float2(0.f, 0.f);
    const float2 wb = okB ? __ldg(P.win0 + T.m * P.sw0 + ra + 1) : make_float2(0.f, 0.f);
    const int chi = min(P.sw1, P.sx1 - T.n * P.hop1);
    const float* ta = tile + (ra - t_r0) * P.tile_w;
    const float2* w1 = P.win1 + T.n * P.sw1;
#pragma unroll
    for (int mm = 0; mm < R; ++mm) {
      const int c = g + G * mm;
      float a = 0.f, b = 0.f;
      if (c < chi && EFF_IN(c, P.tile_w, P.err)) {
        const float2 wc = __ldg(w1 + c);
        if (okA) a = window_weight(wa, wc) * ta[c];
        if (okB) b = window_weight(wb, wc) * ta[P.tile_w + c];
      }
      v[mm] = make_float2(a, b);
    }
    return;
  }
  const bool okA = ra < P.sw0 && i0 < P.sx0;
  const bool okB = ra + 1 < P.sw0 && i0 + 1 < P.sx0;
  const bool okW = !(okA || okB) || EFF_IN(T.m * P.sw0 + ra + (okB ? 1 : 0), P.csf0 * P.sw0, P.err);
  const float2 wa = okA && okW ? __ldg(P.win0 + T.m * P.sw0 + ra) : make_float2(0.f, 0.f);
  const float2 wb = okB && okW ? __ldg(P.win0 + T.m * P.sw0 + ra + 1) : make_float2(0.f, 0.f);
  const int jb = T.n * P.hop1;
  const int chi = min(P.sw1, P.sx1 - jb);
  const long long oa = (long long)i0 * P.sx1 + jb, ob = oa + P.sx1;
  const float2* w1 = P.win1 + T.n * P.sw1;
#pragma unroll
  for (int mm = 0; mm < R; ++mm) {
    const int c = g + G * mm;
    float a = 0.f, b = 0.f;
    if (c < chi && EFF_IN(T.n * P.sw1 + c, P.csf1 * P.sw1, P.err) &&
        (!okA || EFF_IN(oa + c, (long long)P.sx0 * P.sx1, P.err)) &&
        (!okB || EFF_IN(ob + c, (long long)P.sx0 * P.sx1, P.err))) {
      const float2 wc = __ldg(w1 + c);
      if (okA) a = window_weight(wa, wc) * __ldg(T.x + (oa + c));
      if (okB) b = window_weight(wb, wc) * __ldg(T.x + (ob + c));
    }
    v[mm] = make_float2(a, b);
  }
}

// Operand rows (ra, ra+1) packed as re/im, layout A.
template <int N, int KIND>
__device__ __forceinline__ void load_rows(const Params& P, const Patch& T, int ra, int g,
                                          float2 (&v)[FftShape<N>::R], const float* tile = nullptr,
                                          int t_r0 = 0) {
  constexpr int G = FftShape<N>::G;
  constexpr int R = FftShape<N>::R;
  if constexpr (KIND == OPND_RESID) {
    if (T.y_obs && !T.mask) load_resid_rows<N, true, false>(P, T, ra, g, v);
    else if (!T.y_obs && !T.mask) load_resid_rows<N, false, false>(P, T, ra, g, v);
    else if (!T.y_obs) load_resid_rows<N, false, true>(P, T, ra, g, v);
    else load_resid_rows<N, true, true>(P, T, ra, g, v);
  } else if constexpr (KIND == OPND_IMAGE) {
    load_image_rows<N>(P, T, ra, g, v, tile, t_r0);
  } else {
#pragma unroll
    for (int mm = 0; mm < R; ++mm) {
      const int c = g + G * mm;
      v[mm] = make_float2(operand<KIND>(P, T, ra, c), operand<KIND>(P, T, ra + 1, c));
    }
  }
}

// R2C of one pair of rows already in v (layout A), first half: the packed
// transform in v and its Hermitian partners in p (registers only, no frame
// access, so it may run before the cluster's CTAs are known to be running).
template <int N, class TW>
__device__ __forceinline__ void r2c_transform(float2 (&v)[FftShape<N>::R], float2 (&p)[FftShape<N>::R], float2* scr,
                                              const TW& tw, int g, unsigned gmask) {
  fft_fwd<N>(v, g, scr, tw, gmask);
  hermitian_partner<N>(v, p, g, gmask);
}

// Second half: the two half-spectrum rows split from (v, p) into frame rows
// row, row+1 (bins go to the CTA that owns their column).
template <int N, int CL>
__device__ __forceinline__ void r2c_scatter(const float2 (&v)[FftShape<N>::R], const float2 (&p)[FftShape<N>::R],
                                            const Frame<N, CL>& F, int row, int g) {
  constexpr int G = FftShape<N>::G;
  constexpr int R = FftShape<N>::R;
  constexpr int HP = Frame<N, CL>::HP;
  // bins g + G*j of one CTA's range [c W, (c+1) W) are those with j / JW == c
  // (W is a multiple of G); the N/2 bin (j = R/2, lane 0) goes to CTA 0
  constexpr int W = Frame<N, CL>::W;
  constexpr int JW = CL == 1 ? R : R / (2 * CL);
  static_assert(CL == 1 || (R % (2 * CL)) == 0, "cluster split must align with the lane layout");
#pragma unroll
  for (int j = 0; j <= R / 2; ++j) {
    if (j == R / 2 && g != 0) break;
    const int kk = g + G * j;
    const int own = (CL == 1 || j == R / 2) ? 0 : j / JW;
    float2* base = F.part[own];
    const int col = CL == 1 ? kk : (j == R / 2 ? W : kk - own * W);
    float2* rowa = base + row * HP + col;
    if (!EFF_IN((row + 1) * HP + col, F.rows * HP, F.err) || !EFF_IN(col, HP, F.err)) continue;
    rowa[0] = make_float2(0.5f * (v[j].x + p[j].x), 0.5f * (v[j].y - p[j].y));
    rowa[HP] = make_float2(0.5f * (v[j].y + p[j].y), 0.5f * (p[j].x - v[j].x));
  }
}

// C2R of frame rows (ra, ra+1); returns real row ra in .x, ra+1 in .y,
// layout A (register m holds column g + G*m).
template <int N, int CL, class TW>
__device__ __forceinline__ void c2r_unit(const Frame<N, CL>& F, int ra, float2 (&v)[FftShape<N>::R], float2* scr,
                                         const TW& tw, int g, unsigned gmask) {
  constexpr int G = FftShape<N>::G;
  constexpr int R = FftShape<N>::R;
  constexpr int HP = Frame<N, CL>::HP;
#pragma unroll
  for (int j = 0; j < R; ++j) {
    const int kk = g + G * j;
    float2 ya = make_float2(0.f, 0.f), yb = ya;
    const bool lo = j < R / 2 || (j == R / 2 && g == 0);
    const int bin = lo ? kk : N - kk;
    if (EFF_IN((ra + 1) * HP + F.lcol(bin), F.rows * HP, F.err) && EFF_IN(F.lcol(bin), HP, F.err)) {
      const float2* pa = F.at(ra, bin);
      ya = pa[0];
      yb = pa[HP];
      if (!lo) {
        ya.y = -ya.y;
        yb.y = -yb.y;
      }
    }
    v[j] = make_float2(ya.x - yb.y, ya.y + yb.x);
  }
  fft_inv<N>(v, g, scr, tw, gmask);
}

// C2R of the rows at rowa and rowa + out_pitch(N) of this CTA's row-owned
// output block (every bin in local shared memory); layout as c2r_unit.
template <int N, class TW>
__device__ __forceinline__ void c2r_local(const float2* rowa, float2 (&v)[FftShape<N>::R], float2* scr, const TW& tw,
                                          int g, unsigned gmask) {
  constexpr int G = FftShape<N>::G;
  constexpr int R = FftShape<N>::R;
  constexpr int OP3 = out_pitch(N);
#pragma unroll
  for (int j = 0; j < R; ++j) {
    const int kk = g + G * j;
    const bool lo = j < R / 2 || (j == R / 2 && g == 0);
    const int bin = lo ? kk : N - kk;
    float2 ya = rowa[bin], yb = rowa[OP3 + bin];
    if (!lo) {
      ya.y = -ya.y;
      yb.y = -yb.y;
    }
    v[j] = make_float2(ya.x - yb.y, ya.y + yb.x);
  }
  fft_inv<N>(v, g, scr, tw, gmask);
}

// Inverse-transformed column of bin `bin` (dc: bins 0 and N/2 packed as
// re/im) to frame rows [base, base + even(rows)) of the row-owned blocks:
// this CTA's rows by plain stores, the peer's by asynchronous remote stores
// counted on its mbarrier.
template <int N>
__device__ __forceinline__ void store_column_rows(const OutRows<N>& O, int bin, bool dc, int base, int rows, int g,
                                                  const float2 (&v)[FftShape<N>::R]) {
  constexpr int G = FftShape<N>::G;
  constexpr int R = FftShape<N>::R;
  constexpr int OP3 = out_pitch(N);
  const int rows_e = even_up(rows);
  // the peer's block and mbarrier (same offsets in its shared memory)
  const unsigned peer = cluster_addr(smem_addr(O.local), (unsigned)(O.rank ^ 1));
  const unsigned peer_bar = peer + (unsigned)(2 * O.U3 * OP3) * 8u;
#pragma unroll
  for (int mm = 0; mm < R; ++mm) {
    const int r = g + G * mm;
    const int rho = base + r;
    if (r < rows_e && EFF_IN(rho, 4 * O.U3, O.err) && EFF_IN(dc ? N / 2 : bin, N / 2 + 1, O.err)) {
      const bool c1 = (rho >> 1) >= O.U3;
      const int lrow = rho - (c1 ? 2 * O.U3 : 0);
      const float2 a = dc ? make_float2(v[mm].x, 0.f) : v[mm];
      const int b0 = dc ? 0 : bin;
      if (c1 == (O.rank == 1)) {
        float2* q = O.local + lrow * OP3;
        q[b0] = a;
        if (dc) q[N / 2] = make_float2(v[mm].y, 0.f);
      } else {
        const unsigned q = peer + (unsigned)(lrow * OP3) * 8u;
        store_async(q + (unsigned)b0 * 8u, a, peer_bar);
        if (dc) store_async(q + (unsigned)(N / 2) * 8u, make_float2(v[mm].y, 0.f), peer_bar);
      }
    }
  }
}

// Local column `col` (dc: local columns 0 and dcN packed as re/im) of rows
// [base, base+rows), frame pitch HP.
template <int N, int HP>
__device__ __forceinline__ void load_column(const float2* frame, int col, bool dc, int dcN, int base, int rows,
                                            int g, float2 (&v)[FftShape<N>::R], int frows, int* err) {
  constexpr int G = FftShape<N>::G;
  constexpr int R = FftShape<N>::R;
#pragma unroll
  for (int mm = 0; mm < R; ++mm) {
    const int r = g + G * mm;
    if (r < rows && EFF_IN(base + r, frows, err) && EFF_IN(dc ? dcN : col, HP, err)) {
      const float2* row = frame + (base + r) * HP;
      v[mm] = dc ? make_float2(row[0].x, row[dcN].x) : row[col];
    } else {
      v[mm] = make_float2(0.f, 0.f);
    }
  }
}

// Inverse-transformed column to rows [base, base + even(rows)).
template <int N, int HP>
__device__ __forceinline__ void store_column(float2* frame, int col, bool dc, int dcN, int base, int rows,
                                             int g, const float2 (&v)[FftShape<N>::R], int frows, int* err) {
  constexpr int G = FftShape<N>::G;
  constexpr int R = FftShape<N>::R;
  const int rows_e = even_up(rows);
#pragma unroll
  for (int mm = 0; mm < R; ++mm) {
    const int r = g + G * mm;
    if (r < rows_e && EFF_IN(base + r, frows, err) && EFF_IN(dc ? dcN : col, HP, err)) {
      float2* row = frame + (base + r) * HP;
      if (dc) {
        row[0] = make_float2(v[mm].x, 0.f);
        row[dcN] = make_float2(v[mm].y, 0.f);
      } else {
        row[col] = v[mm];
      }
    }
  }
}

// The DC column unit transforms columns 0 and N/2 (both real after the row
// pass) packed as one complex column.  dc_split separates the packed
// spectrum into column 0's (a) and column N/2's (b) and parks both in the
// CTA's DC stash (2N float2, lane-private slots [j*G + g] and
// [N + j*G + g]), so that no third register array is live in the column
// pass.
template <int N>
__device__ __forceinline__ void dc_split(const float2 (&v)[FftShape<N>::R], float2* stash, int g, unsigned gmask) {
  constexpr int G = FftShape<N>::G;
  constexpr int R = FftShape<N>::R;
  float2 p[R];
  hermitian_partner<N>(v, p, g, gmask);
#pragma unroll
  for (int j = 0; j < R; ++j) {
    stash[j * G + g] = make_float2(0.5f * (v[j].x + p[j].x), 0.5f * (v[j].y - p[j].y));
    stash[N + j * G + g] = make_float2(0.5f * (v[j].y + p[j].y), 0.5f * (p[j].x - v[j].x));
  }
}

// Spectrum of column unit u to the cached-spectrum layout [bin][N]: a for
// u != 0, the DC stash's two columns for u == 0.
template <int N>
__device__ __forceinline__ void store_spectrum(float2* __restrict__ dst, int u, int g,
                                               const float2 (&a)[FftShape<N>::R], const float2* stash, int* err) {
  constexpr int G = FftShape<N>::G;
  constexpr int R = FftShape<N>::R;
  if (!EFF_IN(u, N / 2, err)) return;  // bins 0 .. N/2 - 1 (bin N/2 with unit 0)
  float2* c0 = dst + (long long)u * N;
  if (u != 0) {
#pragma unroll
    for (int j = 0; j < R; ++j) c0[g + G * j] = a[j];
  } else {
    float2* cN = dst + (long long)(N / 2) * N;
#pragma unroll
    for (int j = 0; j < R; ++j) {
      c0[g + G * j] = stash[j * G + g];
      cN[g + G * j] = stash[N + j * G + g];
    }
  }
}

// Product of the column spectrum with a cached spectrum bh, packed for one
// inverse transform: u != 0 from a; u == 0 from the DC stash, column 0
// product + i * column N/2 product.  out may alias a.
// Element i of a cached spectrum column, staged in shared memory or in
// global memory (a generic load serves both, so one code path does).
__device__ __forceinline__ float2 spec_at(const float2* c, int i) { return c[i]; }

// c0: the cached spectrum's column of this unit's bin, cN: of bin N/2 (read
// by the DC unit, u == 0, only).
template <int N, bool CONJ>
__device__ __forceinline__ void column_product(const float2 (&a)[FftShape<N>::R], const float2* stash,
                                               const float2* c0, const float2* cN, int u, int g,
                                               float scale, float2 (&out)[FftShape<N>::R]) {
  constexpr int G = FftShape<N>::G;
  constexpr int R = FftShape<N>::R;
  if (u != 0) {
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const float2 s = spec_at(c0, g + G * j);
      out[j] = cscale(CONJ ? cmulc(a[j], s) : cmul(a[j], s), scale);
    }
  } else {
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const float2 s0 = spec_at(c0, g + G * j);
      const float2 sN = spec_at(cN, g + G * j);
      const float2 p0 = CONJ ? cmulc(stash[j * G + g], s0) : cmul(stash[j * G + g], s0);
      const float2 pN = CONJ ? cmulc(stash[N + j * G + g], sN) : cmul(stash[N + j * G + g], sN);
      out[j] = make_float2((p0.x - pN.y) * scale, (p0.y + pN.x) * scale);
    }
  }
}

// Regularised division of the column spectrum y by a cached spectrum s
// (comp_ola_deconv_Kernel, gputools.cu:316-341):
//   z = conj(s) y / (|s|^2 + alpha L + beta),  L(k0, k1) = lap[k1] + lap[k0],
// scaled by `scale`, packed like column_product (u == 0: from the DC stash).
// out may alias a.
template <int N>
__device__ __forceinline__ void column_divide(const float2 (&a)[FftShape<N>::R], const float2* stash,
                                              const float2* c0, const float2* cN, const float* __restrict__ lap,
                                              int u, int g, float alpha, float beta, float scale,
                                              float2 (&out)[FftShape<N>::R]) {
  constexpr int G = FftShape<N>::G;
  constexpr int R = FftShape<N>::R;
  if (u != 0) {
    const float ru = fmaf(alpha, __ldg(lap + u), beta);
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const float2 s = spec_at(c0, g + G * j);
      const float den = fmaf(s.x, s.x, s.y * s.y) + fmaf(alpha, __ldg(lap + g + G * j), ru);
      out[j] = cscale(cmulc(a[j], s), scale / den);
    }
  } else {
    const float r0 = fmaf(alpha, __ldg(lap), beta), rN = fmaf(alpha, __ldg(lap + N / 2), beta);
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const float2 s0 = spec_at(c0, g + G * j);
      const float2 sN = spec_at(cN, g + G * j);
      const float lk = alpha * __ldg(lap + g + G * j);
      const float d0 = fmaf(s0.x, s0.x, s0.y * s0.y) + (lk + r0);
      const float dN = fmaf(sN.x, sN.x, sN.y * sN.y) + (lk + rN);
      const float2 p0 = cscale(cmulc(stash[j * G + g], s0), scale / d0);
      const float2 pN = cscale(cmulc(stash[N + j * G + g], sN), scale / dN);
      out[j] = make_float2(p0.x - pN.y, p0.y + pN.x);
    }
  }
}

// OP_FWD_BOTH, DC unit: s is the PSFs' packed column spectrum (columns 0 and
// N/2 as re/im, transformed like every other column); split it as dc_split
// does, store both PSF spectrum columns, and form the packed product
// (column 0's + i * column N/2's) with the image's split spectrum in the DC
// stash, for one inverse transform.  out may alias the image column.
template <int N>
__device__ __forceinline__ void dc_product_split(const float2 (&s)[FftShape<N>::R], const float2* stash,
                                                 float2* __restrict__ b_out, int g, unsigned gmask, float scale,
                                                 float2 (&out)[FftShape<N>::R]) {
  constexpr int G = FftShape<N>::G;
  constexpr int R = FftShape<N>::R;
  float2 p[R];
  hermitian_partner<N>(s, p, g, gmask);
#pragma unroll
  for (int j = 0; j < R; ++j) {
    const float2 s0 = make_float2(0.5f * (s[j].x + p[j].x), 0.5f * (s[j].y - p[j].y));
    const float2 sN = make_float2(0.5f * (s[j].y + p[j].y), 0.5f * (p[j].x - s[j].x));
    if (b_out) {
      b_out[g + G * j] = s0;
      b_out[(long long)(N / 2) * N + g + G * j] = sN;
    }
    const float2 p0 = cmul(stash[j * G + g], s0);
    const float2 pN = cmul(stash[N + j * G + g], sN);
    out[j] = make_float2((p0.x - pN.y) * scale, (p0.y + pN.x) * scale);
  }
}

// One patch `k` of image `b` through the three phases, on this CTA (and its
// cluster peer when CL = 2).  `cta` / `ncta` number this CTA among the
// CTAs that work on image b (for the loss share).  Every thread of the CTA
// (and of the peer) must call it with the same arguments.
template <int N, int OP, int CL>
__device__ __forceinline__ void eff_patch(const Params& P, int k, long long b, float2* smem, int cta,
                                          int ncta, const CUtensorMap* xmap = nullptr) {
  constexpr int G = FftShape<N>::G;
  constexpr int R = FftShape<N>::R;
  constexpr int A = opnd_a(OP);
  constexpr int HP = frame_pitch(N, CL);
  float2* tw_s = smem;       // N entries (the W_N table; frame 128 keeps each lane's factors in registers)
  float2* frame = smem + N;  // frame_rows(P, OP) * HP
  const int tid = threadIdx.x;
  const int NG = blockDim.x / G;
  const int gid = tid / G, g = tid % G;
  const unsigned gmask = group_mask<N>(tid & 31);

  Frame<N, CL> F;
  F.local = frame;
  F.rows = frame_rows(P, OP);
  F.err = P.err;
  if constexpr (CL == 1) {
    F.rank = 0;
    F.part[0] = frame;
  } else {
    cg::cluster_group cluster = cg::this_cluster();
    F.rank = (int)cluster.block_rank();
#pragma unroll
    for (int r = 0; r < CL; ++r) F.part[r] = cluster.map_shared_rank(frame, r);
  }
  auto phase_sync = [&]() {
    if constexpr (CL == 1) __syncthreads();
    else cg::this_cluster().sync();
  };
  // A cluster barrier that hands over no data (the peers are running / have
  // finished reading this CTA's frame): relaxed arrive, so that it does not
  // wait for this CTA's outstanding global stores and atomics.
  auto cluster_meet = [&]() {
    if constexpr (CL == 1) __syncthreads();
    else asm volatile("barrier.cluster.arrive.relaxed.aligned;\n\tbarrier.cluster.wait.aligned;" ::: "memory");
  };
  // Workers across the cluster for the row passes.
  const int wid = F.rank * NG + gid, NW = CL * NG;

  Patch T;
  T.k = k;
  T.m = T.k / P.csf1;
  T.n = T.k - T.m * P.csf1;
  T.x = P.x ? P.x + b * P.x_bs : nullptr;
  T.f = P.f ? P.f + b * P.f_bs : nullptr;
  T.y = P.y ? P.y + b * P.y_bs : nullptr;
  T.y_obs = P.y_obs ? P.y_obs + b * P.y_bs : nullptr;
  T.mask = P.mask ? P.mask + b * P.y_bs : nullptr;
  const long long spec_patch = (long long)(N / 2 + 1) * N;
  const long long spec_off = b * P.spec_bs + T.k * spec_patch;
  const float2* b0 = P.b0 ? P.b0 + spec_off : nullptr;
  const float2* b1 = P.b1 ? P.b1 + spec_off : nullptr;
  float2* a_out = P.a_out ? P.a_out + spec_off : nullptr;
  float2* b_out = P.b_out ? P.b_out + spec_off : nullptr;

  const int rowsA = opnd_rows(P, A);
  const int baseB = even_up(rowsA);
  float2* scr = frame + frame_rows(P, OP) * HP + gid * FftShape<N>::SCR;
  float2* stash = frame + frame_rows(P, OP) * HP + NG * FftShape<N>::SCR;  // 2N, DC unit only
  // Staged cached spectra: nst columns blocks of SC columns of N + kSpecPad,
  // then the mbarrier their copies complete on.
  constexpr int SC = staged_cols(N, CL);
  constexpr int SP = N + kSpecPad;
  const int nst = staged_specs(P, OP);
  // Row-owned output block (frame-128 pairs): 2 U3 rows of out_pitch(N)
  // bins, then the mbarrier the peer's stores into it complete on.
  constexpr bool kRO = row_owned(N, CL, OP);
  float2* out3 = stash + 2 * N;
  OutRows<N> O;
  O.local = out3;
  O.U3 = phase3_pairs(P, OP, N, CL);
  O.err = P.err;
  O.rank = F.rank;
  unsigned long long* m3 = reinterpret_cast<unsigned long long*>(out3 + 2 * O.U3 * out_pitch(N));
  float2* stage = out3 + (O.U3 ? 2 * O.U3 * out_pitch(N) + 1 : 0);
  stage += (reinterpret_cast<unsigned long long>(stage) & 15ull) ? 1 : 0;
  unsigned long long* sbar = reinterpret_cast<unsigned long long*>(stage + nst * SC * SP);
  // Image tile (operand A = image, a tensor map given): rows [t_r0, t_r0 +
  // tile_rows) of the patch's window -- the rows of the image units this CTA
  // transforms (one round over the cluster: CTA c's 2 NG rows from 2 c NG;
  // else all of them) -- copied by the tensor engine at kernel start.
  float* xtile = nullptr;
  unsigned long long* tbar = nullptr;
  int t_r0 = 0;
  if constexpr (A == OPND_IMAGE) {
    if (xmap && P.tile_rows > 0) {
      unsigned long long a = reinterpret_cast<unsigned long long>(stage + nst * SC * SP + (nst ? 1 : 0));
      a = (a + 127ull) & ~127ull;
      xtile = reinterpret_cast<float*>(a);
      tbar = reinterpret_cast<unsigned long long*>(xtile + ((P.tile_rows * P.tile_w + 1) & ~1));
      t_r0 = P.tile_rows >= even_up(P.sw0) ? 0 : 2 * F.rank * NG;
    }
  }

  // Twiddles: R = 8 (frames 64 and 128) -- this lane's R factors
  // W_N^{g k1} in registers, loaded here with no barrier before the first
  // transform; else the W_N table in shared memory.
  constexpr bool kRegTw = R <= 8;
  const auto tw = [&]() {
    if constexpr (kRegTw) {
      RegTw<R> t;
#pragma unroll
      for (int k1 = 0; k1 < R; ++k1) t.w[k1] = __ldg(P.tw + k1 * G + g);
      return t;
    } else {
      return static_cast<const float2*>(tw_s);
    }
  }();
  // A forward lets the kernel after it (the adjoint of a loss/gradient step)
  // be scheduled now, onto SMs this grid leaves free; a kernel launched that
  // way waits here until its predecessor has finished and its results are
  // visible, before it reads anything that kernel wrote.
  if constexpr (OP == OP_FWD_BOTH || OP == OP_FWD_IMAGE || OP == OP_FWD_PSF)
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  if (P.pdl == 1) asm volatile("griddepcontrol.wait;" ::: "memory");
  if constexpr (!kRegTw)
    for (int i = tid; i < N; i += blockDim.x) tw_s[i] = __ldg(P.tw + i);
  if (nst && tid == 0) mbar_init(sbar, 1);
  // (the peer stores into the row-owned block only after the phase-1 cluster
  // barriers, which follow this initialisation)
  if (kRO && O.U3 && tid == 0) mbar_init(m3, 1);
  if (tbar && tid == 0) {
    mbar_init(tbar, 1);
    mbar_expect_tx(tbar, (unsigned)(P.tile_rows * P.tile_w * sizeof(float)));
    tensor_copy_3d(xtile, xmap, T.n * P.hop1, T.m * P.hop0 + t_r0, (int)b, tbar);
  }
  if (!kRegTw || nst || tbar) __syncthreads();  // the twiddle table / the mbarriers, before the first use
  // Cached spectra this CTA multiplies by in the column pass: its columns of
  // each, copied into shared memory by the bulk-copy engine while the row
  // pass runs (one column per copy, into padded slots).
  if (nst && tid < 32) {
    const int c0 = CL == 1 ? 0 : F.rank * Frame<N, CL>::W;
    const int ncol = CL == 1 ? N / 2 + 1 : Frame<N, CL>::W + (F.rank == 0 ? 1 : 0);
    if (tid == 0) mbar_expect_tx(sbar, (unsigned)(nst * ncol * N * sizeof(float2)));
    __syncwarp();
    const float2* src[2];
    int k = 0;
    if (OP == OP_ADJ || OP == OP_DECONV) {
      if (P.out0) src[k++] = b0;
      if (P.out1) src[k++] = b1;
    } else {
      src[k++] = b0;
    }
    for (int q = tid; q < nst * ncol; q += 32) {
      const int si = q / ncol, l = q - si * ncol;
      // local slot l < W: bin c0 + l; slot W (CTA 0 of a cluster): bin N/2
      const int bin = (CL > 1 && l == Frame<N, CL>::W) ? N / 2 : c0 + l;
      bulk_copy_g2s(stage + (si * SC + l) * SP, src[si] + (long long)bin * N, N * sizeof(float2), sbar);
    }
  }

  // Fused forward of a loss/gradient step: start pulling the observation
  // the adjoint will read into L2 (this CTA's 16-byte-aligned share).
  if constexpr (OP == OP_FWD_BOTH) {
    if (P.pf && tid == 0) {
      const long long per = ((P.pf_bytes + ncta - 1) / ncta + 15) & ~15LL;
      const long long o0 = (long long)cta * per;
      long long n = min(per, P.pf_bytes - o0);
      n &= ~15LL;
      const char* a = P.pf + b * P.pf_bytes + o0;
      if (n > 0 && (reinterpret_cast<unsigned long long>(a) & 15ull) == 0)
        l2_prefetch_bulk(a, (unsigned)n);
    }
  }
  // Kernels that multiply by a cached spectrum in the column pass: pull the
  // columns this CTA owns into L2 now, so that a cold spectrum arrives while
  // the row pass runs (TMA bulk prefetch; a hint, the loads stay as they are).
  if constexpr (OP == OP_FWD_IMAGE || OP == OP_FWD_PSF || OP == OP_ADJ || OP == OP_DECONV) {
    if (!nst && tid < 2) {
      const float2* sp = tid == 0 ? b0 : b1;
      if (sp && (reinterpret_cast<unsigned long long>(sp) & 15ull) == 0) {
        const int c0 = CL == 1 ? 0 : F.rank * Frame<N, CL>::W;
        const int nc = CL == 1 ? N / 2 + 1 : Frame<N, CL>::W;
        l2_prefetch_bulk(sp + (long long)c0 * N, (unsigned)(nc * N * sizeof(float2)));
        if (CL > 1 && F.rank == 0) l2_prefetch_bulk(sp + (long long)(N / 2) * N, (unsigned)(N * sizeof(float2)));
      }
    }
  }
  // Phase 1: row transforms of operand A (and B).  A lane group's first
  // unit is loaded and transformed before the cluster barrier below, so its
  // loads overlap the cluster's start; only its stores into the frames wait.
  {
    const int nA = (rowsA + 1) >> 1;
    const int nB = has_b(OP) ? (P.sf0 + 1) >> 1 : 0;
    // (one loop, so that the transform code exists once: every thread takes
    // the first iteration and meets the barrier there)
    bool first = true;
    bool tile_waited = false;
#pragma unroll 1
    for (int u = wid;; u += NW) {
      float2 v[R], p[R];
      int row = -1;
      if (u < nA + nB) {
        if (u < nA) {
          if (tbar && !tile_waited) {
            tile_waited = true;
            if (!mbar_wait_bounded(tbar, 0)) {
              atomicOr(P.err, kErrCopyTimeout);
              xtile = nullptr;  // this thread reads global memory instead
            }
          }
          load_rows<N, A>(P, T, 2 * u, g, v, xtile, t_r0);
          row = 2 * u;
        } else {
          load_rows<N, OPND_PSF>(P, T, 2 * (u - nA), g, v);
          row = baseB + 2 * (u - nA);
        }
        r2c_transform<N>(v, p, scr, tw, g, gmask);
      }
      if (first) {
        // The peer must not write into this CTA's frame before it is running
        // (and, in a persistent loop, before this CTA has finished the
        // previous patch).
        cluster_meet();
        first = false;
      }
      if (row < 0) break;
      r2c_scatter<N, CL>(v, p, F, row, g);
    }
    // every thread sees the tile copy complete before the CTA can end
    if (tbar && !tile_waited && !mbar_wait_bounded(tbar, 0)) atomicOr(P.err, kErrCopyTimeout);
  }
  phase_sync();

  // This thread's part of the CTA's share of 0.5 ||r||^2 (adjoint with a
  // loss): a contiguous range of pixels per CTA, whole float4s when both
  // planes are 16-byte aligned.
  auto loss_share = [&]() -> float {
    const long long npx = (long long)P.sy0 * P.sy1;
    const bool vec =
        ((reinterpret_cast<unsigned long long>(T.y) | reinterpret_cast<unsigned long long>(T.y_obs)) & 15ull) == 0;
    const long long chunk = vec ? ((npx + ncta - 1) / ncta + 3) & ~3LL : (npx + ncta - 1) / ncta;
    const long long p0 = min(npx, (long long)cta * chunk);
    const long long p1 = min(npx, p0 + chunk);
    const long long q1 = vec ? p0 + ((p1 - p0) & ~3LL) : p0;
    float acc = 0.f;
    const float4* y4 = reinterpret_cast<const float4*>(T.y + p0);
    const float4* o4 = reinterpret_cast<const float4*>(T.y_obs + p0);
    if (T.y_obs) {
      for (int q = tid; q < (int)((q1 - p0) >> 2); q += blockDim.x) {
        const float4 a = __ldg(y4 + q), o = __ldg(o4 + q);
        const float r0 = a.x - o.x, r1 = a.y - o.y, r2 = a.z - o.z, r3 = a.w - o.w;
        acc = fmaf(r0, r0, acc);
        acc = fmaf(r1, r1, acc);
        acc = fmaf(r2, r2, acc);
        acc = fmaf(r3, r3, acc);
      }
      for (long long p = q1 + tid; p < p1; p += blockDim.x) {
        const float r = __ldg(T.y + p) - __ldg(T.y_obs + p);
        acc = fmaf(r, r, acc);
      }
    } else {
      for (int q = tid; q < (int)((q1 - p0) >> 2); q += blockDim.x) {
        const float4 a = __ldg(y4 + q);
        acc = fmaf(a.x, a.x, acc);
        acc = fmaf(a.y, a.y, acc);
        acc = fmaf(a.z, a.z, acc);
        acc = fmaf(a.w, a.w, acc);
      }
      for (long long p = q1 + tid; p < p1; p += blockDim.x) {
        const float r = __ldg(T.y + p);
        acc = fmaf(r, r, acc);
      }
    }
    return acc;
  };
  float loss_acc = 0.f;

  // Phase 2: column transforms, products, inverse column transforms (local).
  constexpr int kUnits = N / 2 / CL;  // column units this CTA owns
  // The bytes the peer's column units will store into this CTA's rows of the
  // row-owned block: every row it owns, the peer's bins (CTA 0: W and bin
  // N/2; CTA 1: W).
  if constexpr (kRO) {
    if (O.U3 && tid == 0) {
      const int rows = max(0, min(2 * (F.rank + 1) * O.U3, 2 * phase3_units(P, OP)) - 2 * F.rank * O.U3);
      const int peer_bins = F.rank == 0 ? N / 4 : N / 4 + 1;
      mbar_expect_tx(m3, (unsigned)(rows * peer_bins * sizeof(float2)));
    }
  }
  constexpr int dcN = Frame<N, CL>::kDcN;
  const float scale = 1.f / (float(N) * float(N));
  // With a spare warp beyond one lane group per unit, the DC unit (CTA 0's
  // local unit 0) runs alone in the last warp and units 1.. on groups 0..: its
  // splits and DC products then serialise no warp of regular units.
  constexpr int GPW = 32 / G;  // lane groups per warp
  const bool dc_alone = F.rank == 0 && NG >= kUnits + GPW;
  const int lu0 = !dc_alone ? gid : (gid == NG - GPW ? 0 : (gid < kUnits - 1 ? gid + 1 : kUnits));
  // the staged spectra must have landed (every thread waits, so none can
  // leave the kernel with a copy into its shared memory still in flight)
  if (nst && !mbar_wait_bounded(sbar, 0)) atomicOr(P.err, kErrCopyTimeout);
  // column of bin u of cached spectrum b (staged: slot si of this CTA) and of bin N/2
  auto spec_col = [&](const float2* b, int si, int lu, int u) -> const float2* {
    if (nst) return EFF_IN(si * SC + lu, nst * SC, P.err) ? stage + (si * SC + lu) * SP : stage;
    return EFF_IN(u, N / 2 + 1, P.err) ? b + (long long)u * N : b;
  };
  auto spec_colN = [&](const float2* b, int si) -> const float2* {
    return nst ? stage + (si * SC + dcN) * SP : b + (long long)(N / 2) * N;
  };
  for (int lu = lu0; lu < kUnits; lu += dc_alone ? kUnits : NG) {
    const int u = F.rank * kUnits + lu;
    const int col = lu;
    // an inverse-transformed column to frame rows [base, base + rows): the
    // row-owned blocks, or this CTA's columns of the frame
    auto put_column = [&](int base, int rows, const float2 (&w)[R]) {
      if constexpr (kRO) store_column_rows<N>(O, u, u == 0, base, rows, g, w);
      else store_column<N, HP>(frame, col, u == 0, dcN, base, rows, g, w, F.rows, F.err);
    };
    // column spectrum of operand A (u == 0: split into the DC stash)
    float2 a[R];
    load_column<N, HP>(frame, col, u == 0, dcN, 0, rowsA, g, a, F.rows, F.err);
    fft_fwd<N>(a, g, scr, tw, gmask);
    if (u == 0) dc_split<N>(a, stash, g, gmask);
    if constexpr (OP == OP_SPEC_IMAGE || OP == OP_SPEC_PSF) {
      store_spectrum<N>(a_out, u, g, a, stash, P.err);
    } else if constexpr (OP == OP_FWD_IMAGE || OP == OP_FWD_PSF) {
      if (a_out) store_spectrum<N>(a_out, u, g, a, stash, P.err);
      column_product<N, false>(a, stash, spec_col(b0, 0, lu, u), spec_colN(b0, 0), u, g, scale, a);
      fft_inv<N>(a, g, scr, tw, gmask);
      put_column(0, P.E0, a);
    } else if constexpr (OP == OP_FWD_BOTH) {
      // a holds the image column spectrum (u == 0: packed, split into the DC
      // stash); transform the PSF column through the same code (u == 0: its
      // columns 0 and N/2 packed the same way) and multiply in place.  The DC
      // unit diverges from the other lane groups of its warp only in the
      // splits and the product.
      if (a_out) store_spectrum<N>(a_out, u, g, a, stash, P.err);
      float2 s[R];
      load_column<N, HP>(frame, col, u == 0, dcN, baseB, P.sf0, g, s, F.rows, F.err);
      fft_fwd<N>(s, g, scr, tw, gmask);
      if (u != 0) {
        if (b_out) store_spectrum<N>(b_out, u, g, s, stash, P.err);
#pragma unroll
        for (int j = 0; j < R; ++j) a[j] = cscale(cmul(a[j], s[j]), scale);
      } else {
        dc_product_split<N>(s, stash, b_out, g, gmask, scale, a);
      }
      fft_inv<N>(a, g, scr, tw, gmask);
      put_column(0, P.E0, a);
    } else {
      // adjoints: output 0 = image (conj F-hat, rows sw0), 1 = PSF (conj X-hat, rows sf0);
      // deconv: the same outputs from the regularised division
#pragma unroll 1
      for (int o = 0; o < 2; ++o) {
        if (o == 0 ? !P.out0 : !P.out1) continue;
        float2 pr[R];
        const float2* bo = o == 0 ? b0 : b1;
        const int si = (o == 1 && P.out0) ? 1 : 0;  // staged order: b0 (when used), then b1
        const float2* c0 = spec_col(bo, si, lu, u);
        const float2* cN = spec_colN(bo, si);
        if constexpr (OP == OP_DECONV)
          column_divide<N>(a, stash, c0, cN, P.lap, u, g, P.alpha, P.beta, scale, pr);
        else
          column_product<N, true>(a, stash, c0, cN, u, g, scale, pr);
        fft_inv<N>(pr, g, scr, tw, gmask);
        const int base = (o == 1 && P.out0) ? even_up(P.sw0) : 0;
        put_column(base, o == 0 ? P.sw0 : P.sf0, pr);
      }
    }
  }
  // Spectrum kernels are done; with a cluster, wait for the peer's local
  // column pass so that a following patch cannot write into its frame early.
  if constexpr (OP == OP_SPEC_IMAGE || OP == OP_SPEC_PSF) {
    if constexpr (CL > 1) cluster_meet();
    return;
  }
  if constexpr (kRO) {
    // this CTA's own rows of the block, then the peer's (its asynchronous
    // stores, counted on m3): no cluster barrier
    __syncthreads();
    if (O.U3 && !mbar_wait_bounded(m3, 0)) atomicOr(P.err, kErrCopyTimeout);
  } else if constexpr (OP == OP_ADJ && CL > 1) {
    // the loss share in the cluster barrier's wait: arrive once this CTA's
    // columns are done, sum the share while the peer finishes, then wait
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
    if (P.loss && (T.y_obs || P.loss_y)) loss_acc = loss_share();
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
  } else {
    phase_sync();
  }
  // the outputs this phase accumulates into are cleared by the kernel before
  if (P.pdl == 2) asm volatile("griddepcontrol.wait;" ::: "memory");
  // Row pairs of this phase: CTA c's contiguous block [c U3, (c+1) U3) over
  // its lane groups (row-owned blocks), else every worker of the cluster in
  // turn.
  const int u3_step = kRO ? NG : NW;
  const int u3_first = kRO ? F.rank * O.U3 + gid : wid;
  auto u3_end = [&](int nu) { return kRO ? min(nu, (F.rank + 1) * O.U3) : nu; };
  auto c2r_pair = [&](int u, float2 (&v)[R]) {
    if constexpr (kRO) {
      const int lr = 2 * (u - F.rank * O.U3);
      if (!EFF_IN(lr + 1, 2 * O.U3, P.err)) {
#pragma unroll
        for (int j = 0; j < R; ++j) v[j] = make_float2(0.f, 0.f);
        return;
      }
      c2r_local<N>(out3 + lr * out_pitch(N), v, scr, tw, g, gmask);
    } else {
      c2r_unit<N, CL>(F, 2 * u, v, scr, tw, g, gmask);
    }
  };

  // Phase 3: inverse row transforms and epilogues.
  if constexpr (OP == OP_FWD_IMAGE || OP == OP_FWD_PSF || OP == OP_FWD_BOTH) {
    float* out = P.out0 + b * P.out0_bs;
    const int i0 = T.m * P.hop0 - P.off0, j0 = T.n * P.hop1 - P.off1;
    const int nu = (P.E0 + 1) >> 1;
    for (int u = u3_first; u < u3_end(nu); u += u3_step) {
      float2 v[R];
      c2r_pair(u, v);
      const int ia = i0 + 2 * u;
      const bool rb = 2 * u + 1 < P.E0;
      // deterministic: the patch's whole E0 x E1 tile, summed by ola_gather
      // (tile row 2u at column c); else the image at row ia, column j0 + c
      const bool tile = P.tiles != nullptr;
      float* dst = tile ? P.tiles + (b * ((long long)P.csf0 * P.csf1) + T.k) * ((long long)P.E0 * P.E1) +
                              (long long)(2 * u) * P.E1
                        : out + (long long)ia * P.sy1 + j0;
      const long long pitch = tile ? P.E1 : P.sy1;
      const bool okA = tile || (ia >= 0 && ia < P.sy0);
      const bool okB = rb && (tile || (ia + 1 >= 0 && ia + 1 < P.sy0));
      const int clo = tile ? 0 : max(0, -j0), chi = tile ? P.E1 : min(P.E1, P.sy1 - j0);
#pragma unroll
      for (int mm = 0; mm < R; ++mm) {
        const int c = g + G * mm;
        if (c >= clo && c < chi) {
          if (okA) ola_put(dst + c, v[mm].x, tile);
          if (okB) ola_put(dst + pitch + c, v[mm].y, tile);
        }
      }
    }
    // out -= sub over this CTA's share of the pixels: the additions commute
    // with the other CTAs' overlap-add, so out ends as the residual
    if (P.sub) {
      const float* sb = P.sub + b * P.y_bs;
      const long long npx = (long long)P.sy0 * P.sy1;
      const bool vec = ((reinterpret_cast<unsigned long long>(out) | reinterpret_cast<unsigned long long>(sb)) &
                        15ull) == 0;
      const long long chunk = vec ? ((npx + ncta - 1) / ncta + 3) & ~3LL : (npx + ncta - 1) / ncta;
      const long long p0 = min(npx, (long long)cta * chunk);
      const long long p1 = min(npx, p0 + chunk);
      const long long q1 = vec ? p0 + ((p1 - p0) & ~3LL) : p0;
      const float4* s4 = reinterpret_cast<const float4*>(sb + p0);
      float4* o4 = reinterpret_cast<float4*>(out + p0);
      for (int q = tid; q < (int)((q1 - p0) >> 2); q += blockDim.x) {
        const float4 s = __ldg(s4 + q);
        atomicAdd(o4 + q, make_float4(-s.x, -s.y, -s.z, -s.w));
      }
      for (long long p = q1 + tid; p < p1; p += blockDim.x) atomicAdd(out + p, -__ldg(sb + p));
    }
  } else if constexpr (OP == OP_ADJ || OP == OP_DECONV) {
    const int n0 = P.out0 ? (P.sw0 + 1) >> 1 : 0;
    const int n1 = P.out1 ? (P.sf0 + 1) >> 1 : 0;
    const int base1 = P.out0 ? even_up(P.sw0) : 0;
    for (int u = u3_first; u < u3_end(n0 + n1); u += u3_step) {
      const bool img = u < n0;
      const int r = img ? 2 * u : 2 * (u - n0);
      float2 v[R];
      c2r_pair(u, v);  // frame rows 2u, 2u + 1 (= img ? r : base1 + r)
      if (img) {
        // image gradient: window, overlap-add into gx (deconv: overlap-add
        // of the sw crop without a window, olaGPU.py:602-607)
        float* out = P.out0 + b * P.out0_bs;
        const int i = T.m * P.hop0 + r;
        const bool rb = r + 1 < P.sw0;
        const float2 wa = __ldg(P.win0 + T.m * P.sw0 + r);
        const float2 wb = rb ? __ldg(P.win0 + T.m * P.sw0 + r + 1) : make_float2(0.f, 0.f);
        // deterministic: the patch's whole sw0 x sw1 tile (row r, column c),
        // summed by ola_gather; else the image at row i, column n hop1 + c
        const bool tile = P.tiles != nullptr;
        float* dst = tile ? P.tiles + (b * ((long long)P.csf0 * P.csf1) + T.k) * ((long long)P.sw0 * P.sw1) +
                                (long long)r * P.sw1
                          : out + (long long)i * P.sx1 + T.n * P.hop1;
        const long long pitch = tile ? P.sw1 : P.sx1;
        const bool okA = tile || i < P.sx0;
        const bool okB = rb && (tile || i + 1 < P.sx0);
        const int chi = tile ? P.sw1 : min(P.sw1, P.sx1 - T.n * P.hop1);
#pragma unroll
        for (int mm = 0; mm < R; ++mm) {
          const int c = g + G * mm;
          if (c < chi) {
            float w0 = 1.f, w1 = 1.f;
            if constexpr (OP == OP_ADJ) {
              const float2 wc = __ldg(P.win1 + T.n * P.sw1 + c);
              w0 = window_weight(wa, wc);
              w1 = window_weight(wb, wc);
            }
            if (okA) ola_put(dst + c, v[mm].x * w0, tile);
            if (okB) ola_put(dst + pitch + c, v[mm].y * w1, tile);
          }
        }
      } else {
        // PSF gradient: crop to sf
        float* out = P.out1 + b * P.out1_bs + (long long)T.k * P.sf0 * P.sf1;
        const bool rb = r + 1 < P.sf0;
#pragma unroll
        for (int mm = 0; mm < R; ++mm) {
          const int c = g + G * mm;
          if (c < P.sf1) {
            out[r * P.sf1 + c] = v[mm].x;
            if (rb) out[(r + 1) * P.sf1 + c] = v[mm].y;
          }
        }
      }
    }
  }
  // Loss of the residual: this CTA's share, summed during the barrier
  // before phase 3 (cluster kernels) or here.
  if constexpr (OP == OP_ADJ) {
    if (P.loss && (T.y_obs || P.loss_y)) {
      const float acc = CL > 1 ? loss_acc : loss_share();
      double d = acc;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
      if (P.loss_part) {
        // deterministic: the CTA's share, warps summed in order, stored for
        // ola_gather (which sums the CTAs' shares in order)
        __shared__ double warp_part[32];
        if ((tid & 31) == 0) warp_part[tid >> 5] = d;
        __syncthreads();
        if (tid == 0) {
          double t = 0.0;
          for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += warp_part[w];
          P.loss_part[b * ncta + cta] = 0.5 * t;
        }
      } else if ((tid & 31) == 0) {
        atomicAdd(P.loss + b, 0.5 * d);
      }
    }
  }
  // Peers read this CTA's frame in phase 3: stay resident until they finish.
  if constexpr (CL > 1) cluster_meet();
  // (a persistent loop initialises the block's mbarrier again for its next patch)
  if constexpr (kRO) {
    if (O.U3 && tid == 0) asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(m3)) : "memory");
  }
}

// Zero the accumulators of the kernel that follows in the same stream (a
// grid-stride share per CTA), so that it needs no memset of its own.
__device__ __forceinline__ void zero_next(const Params& P) {
  const long long cta = (long long)blockIdx.y * gridDim.x + blockIdx.x;
  const long long ncta = (long long)gridDim.x * gridDim.y;
  if (P.zero_f) {
    const long long n = P.zero_nf;
    const bool vec = (reinterpret_cast<unsigned long long>(P.zero_f) & 15ull) == 0;
    const long long n4 = vec ? n / 4 : 0;
    float4* p4 = reinterpret_cast<float4*>(P.zero_f);
    for (long long i = cta * blockDim.x + threadIdx.x; i < n4; i += ncta * blockDim.x)
      p4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (long long i = 4 * n4 + cta * blockDim.x + threadIdx.x; i < n; i += ncta * blockDim.x) P.zero_f[i] = 0.f;
  }
  if (P.zero_d && cta == 0)
    for (int i = threadIdx.x; i < P.zero_nd; i += blockDim.x) P.zero_d[i] = 0.0;
}

// One patch per CTA (CL = 1) or per 2-CTA cluster, images along blockIdx.y.
template <int N, int OP, int CL>
__global__ void __launch_bounds__(max_threads(N))
    eff_kernel(const __grid_constant__ Params P, const __grid_constant__ CUtensorMap xmap) {
  extern __shared__ __align__(128) float2 smem[];
  if constexpr (OP == OP_FWD_BOTH || OP == OP_FWD_IMAGE || OP == OP_FWD_PSF) zero_next(P);
  eff_patch<N, OP, CL>(P, blockIdx.x / CL, blockIdx.y, smem, blockIdx.x, gridDim.x, P.tile_rows > 0 ? &xmap : nullptr);
}

}  // namespace eff
