// Register / sub-warp FFT building blocks for the EFF kernels (sm_103a).
//
// A length-N complex FFT (N = 16*G, G in {4, 8, 16}) is computed by a group of
// G consecutive lanes of one warp, each lane holding 16 values:
//
//   layout "A": lane g, register m  <->  element g + G*m.
//
// Forward:  16-point DFT in registers over m, twiddle by W_N^{g*k1}, exchange
// through a per-group shared-memory scratch so that lane g owns k1 = g + G*t
// (t < 16/G), then G-point DFTs in registers.  The result is again in layout
// A (register j holds X[g + G*j]), so FFT -> pointwise product -> inverse FFT
// needs no reordering.  The inverse runs the same steps backwards with
// conjugate twiddles (unnormalised).
//
// Arithmetic is FP32; the in-register twiddles are exact decimal expansions of
// cos/sin(2*pi*j/16) and the W_N table is computed in FP64 on the host.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace eff {

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

// cos / sin of 2*pi*j/16.
__host__ __device__ constexpr float cos16(int j) {
  constexpr float C1 = 0.92387953251128674f, S1 = 0.38268343236508978f, H = 0.70710678118654752f;
  switch (j & 15) {
    case 0: return 1.f;   case 1: return C1;   case 2: return H;    case 3: return S1;
    case 4: return 0.f;   case 5: return -S1;  case 6: return -H;   case 7: return -C1;
    case 8: return -1.f;  case 9: return -C1;  case 10: return -H;  case 11: return -S1;
    case 12: return 0.f;  case 13: return S1;  case 14: return H;   default: return C1;
  }
}
__host__ __device__ constexpr float sin16(int j) { return cos16(j - 4); }

// v * W where W = exp(-+ 2*pi*i * e16/16) (forward: minus, INV: plus).
template <bool INV>
__device__ __forceinline__ float2 twiddle16(float2 v, int e16) {
  e16 &= 15;
  if (e16 == 0) return v;
  if (e16 == 8) return make_float2(-v.x, -v.y);
  if (e16 == 4) return INV ? make_float2(-v.y, v.x) : make_float2(v.y, -v.x);
  if (e16 == 12) return INV ? make_float2(v.y, -v.x) : make_float2(-v.y, v.x);
  const float c = cos16(e16), s = sin16(e16);
  if (INV) return make_float2(fmaf(v.x, c, -v.y * s), fmaf(v.y, c, v.x * s));
  return make_float2(fmaf(v.x, c, v.y * s), fmaf(v.y, c, -v.x * s));
}

__host__ __device__ constexpr int bitrev(int i, int R) {
  int r = 0;
  for (int b = 1; b < R; b <<= 1) {
    r = (r << 1) | (i & 1);
    i >>= 1;
  }
  return r;
}

// In-register DFT of size R (2..16), natural order in and out.
// Iterative radix-2 decimation in time; every index is a compile-time
// constant after unrolling, so the bit reversal is register renaming.
template <int R, bool INV>
__device__ __forceinline__ void dft(float2 (&a)[R]) {
  float2 b[R];
#pragma unroll
  for (int i = 0; i < R; ++i) b[bitrev(i, R)] = a[i];
#pragma unroll
  for (int len = 2; len <= R; len <<= 1) {
#pragma unroll
    for (int i = 0; i < R; i += len) {
#pragma unroll
      for (int j = 0; j < len / 2; ++j) {
        const float2 u = b[i + j];
        const float2 v = twiddle16<INV>(b[i + j + len / 2], j * (16 / len));
        b[i + j] = cadd(u, v);
        b[i + j + len / 2] = csub(u, v);
      }
    }
  }
#pragma unroll
  for (int i = 0; i < R; ++i) a[i] = b[i];
}

template <int N>
struct FftShape {
  static constexpr int R = 16;          // values per lane
  static constexpr int G = N / 16;      // lanes per transform
  static constexpr int T = R / G;       // k1 values per lane after the exchange
  static constexpr int PAD = 1;         // scratch row padding (bank spread)
  static constexpr int SCR = R * (G + PAD) + 8;  // float2 per group scratch (+8: group offset)
  static_assert(G >= 2 && G <= 16 && (R % G) == 0, "supported N: 32..256");
};

// Forward FFT of length N over a lane group: v in layout A (natural), out in
// layout A (natural).  tw: table [k1*G + g] = W_N^{g*k1}.  scr: this group's
// scratch (FftShape<N>::SCR float2).  mask: the group's lanes.
template <int N>
__device__ __forceinline__ void fft_fwd(float2 (&v)[16], int g, float2* scr, const float2* tw,
                                        unsigned mask) {
  using S = FftShape<N>;
  dft<16, false>(v);
#pragma unroll
  for (int k1 = 1; k1 < 16; ++k1) v[k1] = cmul(v[k1], tw[k1 * S::G + g]);
#pragma unroll
  for (int k1 = 0; k1 < 16; ++k1) scr[k1 * (S::G + S::PAD) + g] = v[k1];
  __syncwarp(mask);
#pragma unroll
  for (int t = 0; t < S::T; ++t) {
    float2 w[S::G];
    const int k1 = g + S::G * t;
#pragma unroll
    for (int n2 = 0; n2 < S::G; ++n2) w[n2] = scr[k1 * (S::G + S::PAD) + n2];
    dft<S::G, false>(w);
#pragma unroll
    for (int k2 = 0; k2 < S::G; ++k2) v[t + S::T * k2] = w[k2];
  }
  __syncwarp(mask);
}

// Inverse (unnormalised) FFT: v in layout A (natural frequency), out layout A.
template <int N>
__device__ __forceinline__ void fft_inv(float2 (&v)[16], int g, float2* scr, const float2* tw,
                                        unsigned mask) {
  using S = FftShape<N>;
#pragma unroll
  for (int t = 0; t < S::T; ++t) {
    float2 w[S::G];
#pragma unroll
    for (int k2 = 0; k2 < S::G; ++k2) w[k2] = v[t + S::T * k2];
    dft<S::G, true>(w);
    const int k1 = g + S::G * t;
#pragma unroll
    for (int n2 = 0; n2 < S::G; ++n2) scr[k1 * (S::G + S::PAD) + n2] = w[n2];
  }
  __syncwarp(mask);
#pragma unroll
  for (int k1 = 0; k1 < 16; ++k1) v[k1] = scr[k1 * (S::G + S::PAD) + g];
  __syncwarp(mask);
#pragma unroll
  for (int k1 = 1; k1 < 16; ++k1) v[k1] = cmulc(v[k1], tw[k1 * S::G + g]);
  dft<16, true>(v);
}

// Value of register j's Hermitian partner: X[N - (g + G*j)] from the lane
// that holds it (lane G-g, register 15-j; lane 0 pairs with itself).
template <int N>
__device__ __forceinline__ void hermitian_partner(const float2 (&v)[16], float2 (&p)[16], int g,
                                                  unsigned mask) {
  using S = FftShape<N>;
  const int src = (S::G - g) & (S::G - 1);
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const float2 s = v[15 - j];
    const float px = __shfl_sync(mask, s.x, src, S::G);
    const float py = __shfl_sync(mask, s.y, src, S::G);
    p[j] = (g == 0) ? v[(16 - j) & 15] : make_float2(px, py);
  }
}

}  // namespace eff
