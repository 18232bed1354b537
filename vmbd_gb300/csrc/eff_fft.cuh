// Register / sub-warp FFT building blocks for the EFF kernels (sm_103a).
//
// A length-N complex FFT (N = R*G: N = 256, 512 with R = 16 values per lane;
// N = 64, 128 with R = 8; N = 192 with R = 24) is computed by a group of G
// consecutive lanes of one warp, each lane holding R values:
//
//   layout "A": lane g, register m  <->  element g + G*m.
//
// Forward:  R-point DFT in registers over m, twiddle by W_N^{g*k1}, exchange
// through a per-group shared-memory scratch so that lane g owns k1 = g + G*t
// (t < R/G), then G-point DFTs in registers.  The result is again in layout
// A (register j holds X[g + G*j]), so FFT -> pointwise product -> inverse FFT
// needs no reordering.  The inverse runs the same steps backwards with
// conjugate twiddles (unnormalised).
//
// Arithmetic is FP32; the in-register twiddles are exact decimal expansions of
// cos/sin(2*pi*j/96) and the W_N table is computed in FP64 on the host.
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

// cos / sin of 2*pi*j/96 (the grid of every in-register twiddle: the radix-2
// stages up to 32 points and the 3 x 8 factorisation of 24).
__host__ __device__ constexpr float cos96_q(int j) {  // j in [0, 24]
  switch (j) {
    case 0: return 1.f;
    case 1: return 0.9978589232386035067f;
    case 2: return 0.9914448613738104111f;
    case 3: return 0.9807852804032304491f;
    case 4: return 0.9659258262890682867f;
    case 5: return 0.9469301294951056642f;
    case 6: return 0.9238795325112867561f;
    case 7: return 0.8968727415326883038f;
    case 8: return 0.8660254037844386467f;
    case 9: return 0.8314696123025452370f;
    case 10: return 0.7933533402912351645f;
    case 11: return 0.7518398074789773964f;
    case 12: return 0.7071067811865475244f;
    case 13: return 0.6593458151000688684f;
    case 14: return 0.6087614290087206394f;
    case 15: return 0.5555702330196022247f;
    case 16: return 0.5f;
    case 17: return 0.4422886902190012819f;
    case 18: return 0.3826834323650897717f;
    case 19: return 0.3214394653031615807f;
    case 20: return 0.2588190451025207623f;
    case 21: return 0.1950903220161282678f;
    case 22: return 0.1305261922200515915f;
    case 23: return 0.0654031292301430668f;
    default: return 0.f;
  }
}
__host__ __device__ constexpr float cos96(int j) {
  j = ((j % 96) + 96) % 96;
  return j <= 24 ? cos96_q(j) : (j <= 48 ? -cos96_q(48 - j) : (j <= 72 ? -cos96_q(j - 48) : cos96_q(96 - j)));
}
__host__ __device__ constexpr float sin96(int j) { return cos96(j - 24); }

// v * W where W = exp(-+ 2*pi*i * e/96) (forward: minus, INV: plus).
template <bool INV>
__device__ __forceinline__ float2 twiddle96(float2 v, int e) {
  e = ((e % 96) + 96) % 96;
  if (e == 0) return v;
  if (e == 48) return make_float2(-v.x, -v.y);
  if (e == 24) return INV ? make_float2(-v.y, v.x) : make_float2(v.y, -v.x);
  if (e == 72) return INV ? make_float2(v.y, -v.x) : make_float2(-v.y, v.x);
  const float c = cos96(e), s = sin96(e);
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

// In-register DFT of a power-of-two size R (2..32), natural order in and
// out: iterative radix-2 decimation in time; every index is a compile-time
// constant after unrolling, so the bit reversal is register renaming.
template <int R, bool INV>
__device__ __forceinline__ void dft_pow2(float2 (&a)[R]) {
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
        const float2 v = twiddle96<INV>(b[i + j + len / 2], j * (96 / len));
        b[i + j] = cadd(u, v);
        b[i + j + len / 2] = csub(u, v);
      }
    }
  }
#pragma unroll
  for (int i = 0; i < R; ++i) a[i] = b[i];
}

// 3-point DFT of (a, b, c) in place.
template <bool INV>
__device__ __forceinline__ void dft3(float2& a, float2& b, float2& c) {
  constexpr float S = 0.86602540378443865f;  // sqrt(3)/2
  const float2 t1 = cadd(b, c), t2 = csub(b, c);
  const float2 m = make_float2(fmaf(-0.5f, t1.x, a.x), fmaf(-0.5f, t1.y, a.y));
  a = cadd(a, t1);
  // forward: X1 = m - i S t2, X2 = m + i S t2 (inverse: the conjugate)
  const float2 n = INV ? make_float2(-S * t2.y, S * t2.x) : make_float2(S * t2.y, -S * t2.x);
  b = cadd(m, n);
  c = csub(m, n);
}

// 24-point DFT: n = 8*n1 + n2, k = k1 + 3*k2 -- DFT-3 over n1 for each n2,
// twiddle W_24^{n2*k1}, DFT-8 over n2 for each k1.
template <bool INV>
__device__ __forceinline__ void dft24(float2 (&a)[24]) {
  float2 y[3][8];
#pragma unroll
  for (int n2 = 0; n2 < 8; ++n2) {
    float2 p = a[n2], q = a[8 + n2], r = a[16 + n2];
    dft3<INV>(p, q, r);
    y[0][n2] = p;
    y[1][n2] = twiddle96<INV>(q, 4 * n2);  // W_24^{n2}
    y[2][n2] = twiddle96<INV>(r, 8 * n2);  // W_24^{2 n2}
  }
#pragma unroll
  for (int k1 = 0; k1 < 3; ++k1) {
    dft_pow2<8, INV>(y[k1]);
#pragma unroll
    for (int k2 = 0; k2 < 8; ++k2) a[k1 + 3 * k2] = y[k1][k2];
  }
}

template <int R, bool INV>
__device__ __forceinline__ void dft(float2 (&a)[R]) {
  if constexpr (R == 24) dft24<INV>(a);
  else dft_pow2<R, INV>(a);
}

// Values each lane holds for a length-N transform (N = 64 and 128: 8 values,
// on 8 and 16 lanes, so that a frame's transforms run on many lanes, each with
// a short dependent chain).
__host__ __device__ constexpr int lane_values(int N) {
  return N % 3 == 0 ? 24 : (N <= 128 ? 8 : 16);
}
// Exchange scratch (float2) of one lane group: R >= G: one R x (G + 1)
// transpose; R = G / 2: a R x (G + 2) transpose, then the N outputs with 8
// padding slots per R*R; +8 spreads the groups of a warp over the banks.
__host__ __device__ constexpr int group_scratch(int N) {
  return lane_values(N) >= N / lane_values(N)
             ? lane_values(N) * (N / lane_values(N) + 1) + 8
             : (lane_values(N) * (N / lane_values(N) + 2) > N + 8 * (N / (lane_values(N) * lane_values(N)))
                    ? lane_values(N) * (N / lane_values(N) + 2)
                    : N + 8 * (N / (lane_values(N) * lane_values(N)))) +
                   8;
}

// A lane's twiddle factors W_N^{g k1} held in registers (frame 128: R = 8 of
// them per lane, loaded once per kernel), or the shared W_N table.
template <int R>
struct RegTw {
  float2 w[R];
};
template <int G>
__device__ __forceinline__ float2 tw_at(const float2* t, int k1, int g) {
  return t[k1 * G + g];
}
template <int G, int R>
__device__ __forceinline__ float2 tw_at(const RegTw<R>& t, int k1, int) {
  return t.w[k1];
}

template <int N>
struct FftShape {
  static constexpr int R = lane_values(N);          // values per lane
  static constexpr int G = N / R;                    // lanes per transform
  static constexpr int T = R / G;                    // k1 values per lane after the exchange (R >= G)
  static constexpr int PAD = 1;                      // scratch row padding (bank spread, R >= G)
  static constexpr int SCR = group_scratch(N);       // float2 per group scratch
  static_assert(G >= 2 && G <= 32 && ((R % G) == 0 || 2 * R == G) && (G & (G - 1)) == 0,
                "supported N: 32..512, 192");
};

// Forward FFT for R = G / 2 (N = 128: 8 values on 16 lanes; N = 512: 16
// values on 32 lanes).  With
// n = g + G m and k = k1 + R k2: an R-point DFT over m in registers, the
// twiddle W_N^{g k1}, then for each k1 a G-point DFT over g, which lanes
// 2 k1 (even g) and 2 k1 + 1 (odd g) share: after a transpose through the
// scratch each takes an R-point DFT of its half, the odd one twiddles by
// W_G^{k2}, and one exchange of partners (shuffle) gives the butterfly --
// the even lane then holds X[k1 + R k2], k2 < R, the odd one k2 >= R.  A
// second pass through the scratch restores layout A.
template <int N, class TW>
__device__ __forceinline__ void fft_fwd_half(float2 (&v)[FftShape<N>::R], int g, float2* scr, const TW& tw,
                                             unsigned mask) {
  using S = FftShape<N>;
  constexpr int R = S::R;
  constexpr int G = S::G;
  static_assert(2 * R == G, "R = G / 2");
  constexpr int P1 = G + 2;  // transpose row pitch (conflict-free reads of the odd/even halves)
  dft<R, false>(v);
#pragma unroll
  for (int k1 = 1; k1 < R; ++k1) v[k1] = cmul(v[k1], tw_at<G>(tw, k1, g));
#pragma unroll
  for (int k1 = 0; k1 < R; ++k1) scr[k1 * P1 + g] = v[k1];
  __syncwarp(mask);
  const int p = g >> 1, h = g & 1;
#pragma unroll
  for (int j = 0; j < R; ++j) v[j] = scr[p * P1 + 2 * j + h];
  __syncwarp(mask);
  dft<R, false>(v);
  if (h) {
#pragma unroll
    for (int k = 1; k < R; ++k) v[k] = twiddle96<false>(v[k], k * (96 / G));  // W_G^k
  }
#pragma unroll
  for (int k = 0; k < R; ++k) {
    const float ox = __shfl_xor_sync(mask, v[k].x, 1, G);
    const float oy = __shfl_xor_sync(mask, v[k].y, 1, G);
    // even lane: E + W O; odd lane: E - W O (its own value is W O)
    v[k] = h ? make_float2(ox - v[k].x, oy - v[k].y) : make_float2(v[k].x + ox, v[k].y + oy);
  }
  // X[p + R (k + R h)] -> the scratch (8 padding slots per R*R, so that the
  // two halves h of a half-warp land on different banks), layout A back out
#pragma unroll
  for (int k = 0; k < R; ++k) {
    const int n = p + R * k + R * R * h;
    scr[n + (n / (R * R)) * 8] = v[k];
  }
  __syncwarp(mask);
#pragma unroll
  for (int m = 0; m < R; ++m) {
    const int n = g + G * m;
    v[m] = scr[n + (n / (R * R)) * 8];
  }
  __syncwarp(mask);
}

// Forward FFT of length N over a lane group: v in layout A (natural), out in
// layout A (natural).  tw: table [k1*G + g] = W_N^{g*k1}.  scr: this group's
// scratch (FftShape<N>::SCR float2).  mask: the group's lanes.
template <int N, class TW>
__device__ __forceinline__ void fft_fwd(float2 (&v)[FftShape<N>::R], int g, float2* scr, const TW& tw,
                                        unsigned mask) {
  using S = FftShape<N>;
  constexpr int R = S::R;
  if constexpr (R < S::G) {
    fft_fwd_half<N>(v, g, scr, tw, mask);
  } else {
    dft<R, false>(v);
#pragma unroll
    for (int k1 = 1; k1 < R; ++k1) v[k1] = cmul(v[k1], tw_at<S::G>(tw, k1, g));
#pragma unroll
    for (int k1 = 0; k1 < R; ++k1) scr[k1 * (S::G + S::PAD) + g] = v[k1];
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
}

// Inverse (unnormalised) FFT: v in layout A (natural frequency), out layout A.
// (R = G / 2: conj(FFT(conj(v))).)
template <int N, class TW>
__device__ __forceinline__ void fft_inv(float2 (&v)[FftShape<N>::R], int g, float2* scr, const TW& tw,
                                        unsigned mask) {
  using S = FftShape<N>;
  constexpr int R = S::R;
  if constexpr (R < S::G) {
#pragma unroll
    for (int j = 0; j < R; ++j) v[j].y = -v[j].y;
    fft_fwd_half<N>(v, g, scr, tw, mask);
#pragma unroll
    for (int j = 0; j < R; ++j) v[j].y = -v[j].y;
  } else {
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
    for (int k1 = 0; k1 < R; ++k1) v[k1] = scr[k1 * (S::G + S::PAD) + g];
    __syncwarp(mask);
#pragma unroll
    for (int k1 = 1; k1 < R; ++k1) v[k1] = cmulc(v[k1], tw_at<S::G>(tw, k1, g));
    dft<R, true>(v);
  }
}

// Value of register j's Hermitian partner: X[N - (g + G*j)] from the lane
// that holds it (lane G-g, register R-1-j; lane 0 pairs with itself).
template <int N>
__device__ __forceinline__ void hermitian_partner(const float2 (&v)[FftShape<N>::R], float2 (&p)[FftShape<N>::R],
                                                  int g, unsigned mask) {
  using S = FftShape<N>;
  constexpr int R = S::R;
  const int src = (S::G - g) & (S::G - 1);
#pragma unroll
  for (int j = 0; j < R; ++j) {
    const float2 s = v[R - 1 - j];
    const float px = __shfl_sync(mask, s.x, src, S::G);
    const float py = __shfl_sync(mask, s.y, src, S::G);
    p[j] = (g == 0) ? v[(R - j) % R] : make_float2(px, py);
  }
}

}  // namespace eff
