// Fused EFF kernels: one CTA per patch (blockIdx.x) and image (blockIdx.y).
//
// Every kernel runs the same three phases over an N x N frame (N = 64/128/256,
// a power of two >= sw + sf - 1 in both dims) held as a half spectrum
// (N/2+1 bins per row) in shared memory:
//
//  1. row pass (R2C): pairs of real operand rows are read straight from HBM
//     (windowed image patch, PSF, or the output-side image for the adjoints),
//     packed as one complex row, transformed, and split into two half-spectrum
//     rows.
//  2. column pass: each lane group takes one column (columns 0 and N/2, both
//     real after the row pass, share one complex transform), transforms it,
//     optionally stores it as a cached spectrum, multiplies it by the cached
//     spectrum of the other operand (conjugated for the adjoints) and inverse
//     transforms it, all in registers; only the rows the epilogue needs go
//     back to shared memory.
//  3. row pass (C2R): pairs of half-spectrum rows are inverse transformed as
//     one complex row; the epilogue overlap-adds into the output image with
//     fp32 atomics (forward: full-convolution extent, cropped by mode; image
//     adjoint: windowed, patch extent) or stores the PSF gradient.
//
// Reference semantics: OlaGPU.cnv / OlaGPU.cnvtp, olaGPU.py:170-311.
#pragma once
#include "eff_fft.cuh"

namespace eff {

enum Op : int {
  OP_SPEC_IMAGE = 0,  // X-hat of the windowed patches (OlaGPU X object, olaGPU.py:147-157)
  OP_SPEC_PSF = 1,    // F-hat of the PSFs (OlaGPU F object, olaGPU.py:142-157)
  OP_FWD_IMAGE = 2,   // y = F x   (F.cnv(x), olaGPU.py:200-257)
  OP_FWD_PSF = 3,     // y = X f   (X.cnv(f), olaGPU.py:188-193, 219-257)
  OP_ADJ = 4,         // F^T y and/or X^T y (cnvtp, olaGPU.py:261-311)
};

struct Params {
  int sx0, sx1, sf0, sf1, csf0, csf1, sw0, sw1, hop0, hop1;
  int sy0, sy1, off0, off1, E0, E1;
  int lo0, hi0, lo1, hi1;  // adjoint input window inside a frame
  const float* x;          // image [sx0, sx1]
  const float* f;          // PSFs [K, sf0, sf1]
  const float* y;          // output-side image [sy0, sy1] (adjoint input)
  const float2* b0;        // cached spectrum: F-hat (fwd image / adj image) or X-hat (fwd psf)
  const float2* b1;        // cached spectrum: X-hat (adj psf)
  float2* a_out;           // spectrum of this kernel's operand (optional)
  float* out0;             // y (forward) or gx (image adjoint)
  float* out1;             // gf (PSF adjoint)
  const float2* win0;      // window factors (alpha, gamma) [csf0, sw0]
  const float2* win1;      // window factors (alpha, gamma) [csf1, sw1]
  const float2* tw;        // W_N table [16*G]
  long long x_bs, f_bs, y_bs, spec_bs, out0_bs, out1_bs;  // per-image strides
};

__host__ __device__ constexpr int frame_pitch(int N) { return N / 2 + 1; }

template <int N>
__device__ __forceinline__ unsigned group_mask(int lane) {
  constexpr int G = FftShape<N>::G;
  return G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
}

// Window weight ws[k=(m,n)][r][c] from the per-dim (alpha, gamma) tables:
// alpha*alpha' inside the image, gamma*gamma' = 1/(patches covering the
// pixel) on the outermost rows/columns that only zero-valued window samples
// reach (alpha < 0 marks them).  That is the reference's partition of unity
// w / chop(ola(w)) with w floored at 1e-16 (imagetools.py:341, 437-445).
__device__ __forceinline__ float window_weight(float2 u, float2 v) {
  return (u.x < 0.f || v.x < 0.f) ? u.y * v.y : u.x * v.x;
}

// Operand value at frame position (r, c) of patch (m, n) / index k.
template <int OP>
__device__ __forceinline__ float operand(const Params& P, const float* x, const float* f,
                                         const float* y, int m, int n, int k, int r, int c) {
  if constexpr (OP == OP_SPEC_IMAGE || OP == OP_FWD_IMAGE) {
    if (r >= P.sw0 || c >= P.sw1) return 0.f;
    const int i = m * P.hop0 + r, j = n * P.hop1 + c;
    if (i >= P.sx0 || j >= P.sx1) return 0.f;
    return window_weight(__ldg(P.win0 + m * P.sw0 + r), __ldg(P.win1 + n * P.sw1 + c)) *
           __ldg(x + (long long)i * P.sx1 + j);
  } else if constexpr (OP == OP_SPEC_PSF || OP == OP_FWD_PSF) {
    if (r >= P.sf0 || c >= P.sf1) return 0.f;
    return __ldg(f + ((long long)k * P.sf0 + r) * P.sf1 + c);
  } else {
    if (r < P.lo0 || r >= P.hi0 || c < P.lo1 || c >= P.hi1) return 0.f;
    const int i = m * P.hop0 + r - P.off0, j = n * P.hop1 + c - P.off1;
    if (i < 0 || j < 0 || i >= P.sy0 || j >= P.sy1) return 0.f;
    return __ldg(y + (long long)i * P.sy1 + j);
  }
}

template <int OP>
__device__ __forceinline__ int operand_rows(const Params& P) {
  if constexpr (OP == OP_SPEC_IMAGE || OP == OP_FWD_IMAGE) return P.sw0;
  else if constexpr (OP == OP_SPEC_PSF || OP == OP_FWD_PSF) return P.sf0;
  else return P.E0;
}

// Phase 1: real operand rows -> half-spectrum rows [0, even(rows)).
template <int N, int OP>
__device__ __forceinline__ void row_r2c(const Params& P, const float* x, const float* f,
                                        const float* y, int m, int n, int k, float2* frame,
                                        float2* scr, const float2* tw, int gid, int NG, int g,
                                        unsigned gmask) {
  constexpr int G = FftShape<N>::G;
  constexpr int HP = frame_pitch(N);
  const int rows = operand_rows<OP>(P);
  const int nunits = (rows + 1) >> 1;
  for (int u = gid; u < nunits; u += NG) {
    const int ra = 2 * u, rb = ra + 1;
    float2 v[16];
#pragma unroll
    for (int mm = 0; mm < 16; ++mm) {
      const int c = g + G * mm;
      v[mm] = make_float2(operand<OP>(P, x, f, y, m, n, k, ra, c),
                          operand<OP>(P, x, f, y, m, n, k, rb, c));
    }
    fft_fwd<N>(v, g, scr, tw, gmask);
    float2 p[16];
    hermitian_partner<N>(v, p, g, gmask);
#pragma unroll
    for (int j = 0; j <= 8; ++j) {
      if (j == 8 && g != 0) break;
      const int kk = g + G * j;
      frame[ra * HP + kk] = make_float2(0.5f * (v[j].x + p[j].x), 0.5f * (v[j].y - p[j].y));
      frame[rb * HP + kk] = make_float2(0.5f * (v[j].y + p[j].y), 0.5f * (p[j].x - v[j].x));
    }
  }
}

// Phase 3: half-spectrum rows [base, base+nrows) -> real rows, fed to epi(r, c, value).
template <int N, class Epi>
__device__ __forceinline__ void row_c2r(float2* frame, int base, int nrows, int ncols,
                                        float2* scr, const float2* tw, int gid, int NG, int g,
                                        unsigned gmask, Epi epi) {
  constexpr int G = FftShape<N>::G;
  constexpr int HP = frame_pitch(N);
  const int nunits = (nrows + 1) >> 1;
  for (int u = gid; u < nunits; u += NG) {
    const int ra = base + 2 * u, rb = ra + 1;
    float2 v[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const int kk = g + G * j;
      float2 ya, yb;
      if (j < 8 || (j == 8 && g == 0)) {
        ya = frame[ra * HP + kk];
        yb = frame[rb * HP + kk];
      } else {
        ya = frame[ra * HP + (N - kk)];
        yb = frame[rb * HP + (N - kk)];
        ya.y = -ya.y;
        yb.y = -yb.y;
      }
      v[j] = make_float2(ya.x - yb.y, ya.y + yb.x);
    }
    fft_inv<N>(v, g, scr, tw, gmask);
    const bool has_b = (2 * u + 1) < nrows;
#pragma unroll
    for (int mm = 0; mm < 16; ++mm) {
      const int c = g + G * mm;
      if (c < ncols) {
        epi(2 * u, c, v[mm].x);
        if (has_b) epi(2 * u + 1, c, v[mm].y);
      }
    }
  }
}

// Load column unit u (u == 0: columns 0 and N/2 packed) of rows [0, rows).
template <int N>
__device__ __forceinline__ void load_column(const float2* frame, int u, int rows, int g,
                                            float2 (&v)[16]) {
  constexpr int G = FftShape<N>::G;
  constexpr int HP = frame_pitch(N);
#pragma unroll
  for (int mm = 0; mm < 16; ++mm) {
    const int r = g + G * mm;
    if (r < rows) {
      if (u == 0) v[mm] = make_float2(frame[r * HP].x, frame[r * HP + N / 2].x);
      else v[mm] = frame[r * HP + u];
    } else {
      v[mm] = make_float2(0.f, 0.f);
    }
  }
}

// Store an inverse-transformed column to rows [base, base + even(rows)).
template <int N>
__device__ __forceinline__ void store_column(float2* frame, int u, int base, int rows, int g,
                                             const float2 (&v)[16]) {
  constexpr int G = FftShape<N>::G;
  constexpr int HP = frame_pitch(N);
  const int rows_e = (rows + 1) & ~1;
#pragma unroll
  for (int mm = 0; mm < 16; ++mm) {
    const int r = g + G * mm;
    if (r < rows_e) {
      float2* row = frame + (base + r) * HP;
      if (u == 0) {
        row[0] = make_float2(v[mm].x, 0.f);
        row[N / 2] = make_float2(v[mm].y, 0.f);
      } else {
        row[u] = v[mm];
      }
    }
  }
}

// Spectrum of column unit u: two columns for u == 0.
template <int N>
struct ColSpec {
  float2 a[16];  // column u (u == 0: column 0)
  float2 b[16];  // u == 0: column N/2
};

// Pointwise product of an operand column spectrum with a cached spectrum,
// packed for one inverse transform; scale = 1/N^2.
template <int N, bool CONJ>
__device__ __forceinline__ void column_product(const ColSpec<N>& s, const float2* __restrict__ bh,
                                               int u, int g, float scale, float2 (&out)[16]) {
  constexpr int G = FftShape<N>::G;
  const float2* c0 = bh + (long long)u * N;
  if (u != 0) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const float2 b = __ldg(c0 + g + G * j);
      out[j] = cscale(CONJ ? cmulc(s.a[j], b) : cmul(s.a[j], b), scale);
    }
  } else {
    const float2* cN = bh + (long long)(N / 2) * N;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const float2 b0 = __ldg(c0 + g + G * j);
      const float2 bN = __ldg(cN + g + G * j);
      const float2 p0 = CONJ ? cmulc(s.a[j], b0) : cmul(s.a[j], b0);
      const float2 pN = CONJ ? cmulc(s.b[j], bN) : cmul(s.b[j], bN);
      out[j] = make_float2((p0.x - pN.y) * scale, (p0.y + pN.x) * scale);
    }
  }
}

template <int N>
__device__ __forceinline__ void store_spectrum(float2* __restrict__ dst, const ColSpec<N>& s, int u,
                                               int g) {
  constexpr int G = FftShape<N>::G;
  float2* c0 = dst + (long long)u * N;
#pragma unroll
  for (int j = 0; j < 16; ++j) c0[g + G * j] = s.a[j];
  if (u == 0) {
    float2* cN = dst + (long long)(N / 2) * N;
#pragma unroll
    for (int j = 0; j < 16; ++j) cN[g + G * j] = s.b[j];
  }
}

template <int N>
__device__ __forceinline__ void column_spectrum(const float2* frame, int u, int rows, int g,
                                                float2* scr, const float2* tw, unsigned gmask,
                                                ColSpec<N>& s) {
  load_column<N>(frame, u, rows, g, s.a);
  fft_fwd<N>(s.a, g, scr, tw, gmask);
  if (u == 0) {
    // Columns 0 and N/2 are real: split X = A + iB into A and B.
    float2 p[16];
    hermitian_partner<N>(s.a, p, g, gmask);
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const float2 v = s.a[j];
      s.a[j] = make_float2(0.5f * (v.x + p[j].x), 0.5f * (v.y - p[j].y));
      s.b[j] = make_float2(0.5f * (v.y + p[j].y), 0.5f * (p[j].x - v.x));
    }
  }
}

template <int N, int OP>
__global__ void __launch_bounds__(256) eff_kernel(Params P) {
  constexpr int G = FftShape<N>::G;
  constexpr int HP = frame_pitch(N);
  extern __shared__ __align__(16) float2 smem[];
  float2* tw = smem;                 // N entries
  float2* frame = smem + N;          // rows * HP (rows set by the host)
  const int tid = threadIdx.x;
  const int NG = blockDim.x / G;
  const int gid = tid / G, g = tid % G;
  const unsigned gmask = group_mask<N>(tid & 31);

  const int k = blockIdx.x;
  const int m = k / P.csf1, n = k - (k / P.csf1) * P.csf1;
  const long long b = blockIdx.y;
  const float* x = P.x ? P.x + b * P.x_bs : nullptr;
  const float* f = P.f ? P.f + b * P.f_bs : nullptr;
  const float* y = P.y ? P.y + b * P.y_bs : nullptr;
  const long long spec_patch = (long long)(N / 2 + 1) * N;
  const float2* b0 = P.b0 ? P.b0 + b * P.spec_bs + k * spec_patch : nullptr;
  const float2* b1 = P.b1 ? P.b1 + b * P.spec_bs + k * spec_patch : nullptr;
  float2* a_out = P.a_out ? P.a_out + b * P.spec_bs + k * spec_patch : nullptr;

  // Frame rows in use (same formula as the host's shared-memory sizing).
  int rows_alloc;
  if constexpr (OP == OP_SPEC_IMAGE || OP == OP_SPEC_PSF) rows_alloc = (operand_rows<OP>(P) + 1) & ~1;
  else if constexpr (OP == OP_FWD_IMAGE || OP == OP_FWD_PSF) rows_alloc = (P.E0 + 1) & ~1;
  else {
    const int r0 = P.out0 ? ((P.sw0 + 1) & ~1) : 0;
    const int r1 = P.out1 ? ((P.sf0 + 1) & ~1) : 0;
    rows_alloc = max((P.E0 + 1) & ~1, r0 + r1);
  }
  float2* scr = frame + rows_alloc * HP + gid * FftShape<N>::SCR;

  for (int i = tid; i < N; i += blockDim.x) tw[i] = __ldg(P.tw + i);
  __syncthreads();

  row_r2c<N, OP>(P, x, f, y, m, n, k, frame, scr, tw, gid, NG, g, gmask);
  __syncthreads();

  const int rowsA = operand_rows<OP>(P);
  const float scale = 1.f / (float(N) * float(N));
  for (int u = gid; u < N / 2; u += NG) {
    ColSpec<N> s;
    column_spectrum<N>(frame, u, rowsA, g, scr, tw, gmask, s);
    if constexpr (OP == OP_SPEC_IMAGE || OP == OP_SPEC_PSF) {
      store_spectrum<N>(a_out, s, u, g);
    } else if constexpr (OP == OP_FWD_IMAGE || OP == OP_FWD_PSF) {
      if (a_out) store_spectrum<N>(a_out, s, u, g);
      float2 pr[16];
      column_product<N, false>(s, b0, u, g, scale, pr);
      fft_inv<N>(pr, g, scr, tw, gmask);
      store_column<N>(frame, u, 0, P.E0, g, pr);
    } else {
      if (P.out0) {
        float2 pr[16];
        column_product<N, true>(s, b0, u, g, scale, pr);
        fft_inv<N>(pr, g, scr, tw, gmask);
        store_column<N>(frame, u, 0, P.sw0, g, pr);
      }
      if (P.out1) {
        float2 pr[16];
        column_product<N, true>(s, b1, u, g, scale, pr);
        fft_inv<N>(pr, g, scr, tw, gmask);
        store_column<N>(frame, u, P.out0 ? ((P.sw0 + 1) & ~1) : 0, P.sf0, g, pr);
      }
    }
  }
  if constexpr (OP == OP_SPEC_IMAGE || OP == OP_SPEC_PSF) return;
  __syncthreads();

  if constexpr (OP == OP_FWD_IMAGE || OP == OP_FWD_PSF) {
    float* out = P.out0 + b * P.out0_bs;
    const int i0 = m * P.hop0 - P.off0, j0 = n * P.hop1 - P.off1;
    row_c2r<N>(frame, 0, P.E0, P.E1, scr, tw, gid, NG, g, gmask, [&](int r, int c, float val) {
      const int i = i0 + r, j = j0 + c;
      if (i >= 0 && j >= 0 && i < P.sy0 && j < P.sy1) atomicAdd(out + (long long)i * P.sy1 + j, val);
    });
  } else if constexpr (OP == OP_ADJ) {
    if (P.out0) {
      float* out = P.out0 + b * P.out0_bs;
      const float2* w0 = P.win0 + m * P.sw0;
      const float2* w1 = P.win1 + n * P.sw1;
      const int i0 = m * P.hop0, j0 = n * P.hop1;
      row_c2r<N>(frame, 0, P.sw0, P.sw1, scr, tw, gid, NG, g, gmask, [&](int r, int c, float val) {
        const int i = i0 + r, j = j0 + c;
        if (i < P.sx0 && j < P.sx1)
          atomicAdd(out + (long long)i * P.sx1 + j, val * window_weight(__ldg(w0 + r), __ldg(w1 + c)));
      });
    }
    if (P.out1) {
      float* out = P.out1 + b * P.out1_bs + (long long)k * P.sf0 * P.sf1;
      row_c2r<N>(frame, P.out0 ? ((P.sw0 + 1) & ~1) : 0, P.sf0, P.sf1, scr, tw, gid, NG, g, gmask,
                 [&](int r, int c, float val) { out[r * P.sf1 + c] = val; });
    }
  }
}

}  // namespace eff
