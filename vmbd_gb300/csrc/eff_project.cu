// PSF projections (one CTA per PSF) and the basis dot product.
//
// clip_normalize: the reference's PSF constraint -- non-negativity (L-BFGS-B
//   bounds, olaGPU.py:404-411; cliplower_GPU, gputools.py:478-486) then
//   per-PSF unit sum when the sum exceeds 1e-6 (normalize,
//   gputools.py:1025-1044, which the reference runs on the host).
// simplex: Euclidean projection onto {f >= 0, sum f = 1} by Michelot's
//   active-set iteration (Michelot 1986): tau = (sum_{f_i > tau} f_i - 1) /
//   #{f_i > tau}, repeated until the active set stops shrinking (at most n
//   rounds; tau never decreases), then f = max(f - tau, 0).  Same result as
//   the sort-based method of Duchi et al. 2008.
// basis_project: w[b] = <fs, basis_b>, what projection.cu:3-27 computes for a
//   correct block/column indexing.
// All reductions are fixed-order trees, so results are run-to-run identical.
#include <cuda_runtime.h>

namespace eff {

constexpr int kProjThreads = 256;

// Deterministic block sum of (a, b); every thread gets the totals.
__device__ __forceinline__ float2 block_sum2(float a, float b, float2* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = make_float2(a, b);
  __syncthreads();
  const int nw = blockDim.x >> 5;
  float2 t = l < nw ? red[l] : make_float2(0.f, 0.f);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    t.x += __shfl_xor_sync(0xffffffffu, t.x, o);
    t.y += __shfl_xor_sync(0xffffffffu, t.y, o);
  }
  return t;
}

__global__ void __launch_bounds__(kProjThreads) clip_normalize_kernel(float* f, int n) {
  __shared__ float2 red[32];
  float* p = f + (long long)blockIdx.x * n;
  float s = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const float v = fmaxf(p[i], 0.f);
    p[i] = v;
    s += v;
  }
  const float tot = block_sum2(s, 0.f, red).x;
  if (tot > 1e-6f) {
    const float inv = 1.f / tot;
    for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = p[i] * inv;
  }
}

__global__ void __launch_bounds__(kProjThreads) simplex_kernel(float* f, int n) {
  __shared__ float2 red[32];
  float* p = f + (long long)blockIdx.x * n;
  float s = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += p[i];
  float2 t = block_sum2(s, 0.f, red);
  float tau = (t.x - 1.f) / float(n);
  int count = n;
  for (int it = 0; it <= n; ++it) {
    float ss = 0.f, cc = 0.f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const float v = p[i];
      if (v > tau) {
        ss += v;
        cc += 1.f;
      }
    }
    t = block_sum2(ss, cc, red);
    const int c = int(t.y + 0.5f);
    if (c == 0) break;
    const float tn = (t.x - 1.f) / t.y;
    if (c == count) {
      tau = tn;
      break;
    }
    count = c;
    tau = tn;
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = fmaxf(p[i] - tau, 0.f);
}

__global__ void __launch_bounds__(kProjThreads) basis_project_kernel(const float* fs, const float* basis,
                                                                     float* w, int n) {
  __shared__ float2 red[32];
  const float* bp = basis + (long long)blockIdx.x * n;
  float s = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s = fmaf(__ldg(fs + i), __ldg(bp + i), s);
  const float tot = block_sum2(s, 0.f, red).x;
  if (threadIdx.x == 0) w[blockIdx.x] = tot;
}

cudaError_t launch_project(float* f, int K, int n, int mode, cudaStream_t st) {
  if (mode == 0) clip_normalize_kernel<<<K, kProjThreads, 0, st>>>(f, n);
  else simplex_kernel<<<K, kProjThreads, 0, st>>>(f, n);
  return cudaGetLastError();
}

cudaError_t launch_basis_project(const float* fs, const float* basis, float* w, int nb, int n,
                                 cudaStream_t st) {
  basis_project_kernel<<<nb, kProjThreads, 0, st>>>(fs, basis, w, n);
  return cudaGetLastError();
}

}  // namespace eff

namespace eff {

// Edge taper in place (edgetaper.cu:6-31 via edgetaper_gpu,
// gputools.py:643-673): rows i < hy are scaled by wy[i], rows
// i > rows-1-hy by wy[rows-1-i], likewise columns with wx; the interior is
// untouched.  Both images of a batch share the tables.
__global__ void edgetaper_kernel(float* im, int rows, int cols, const float* __restrict__ wy, int hy,
                                 const float* __restrict__ wx, int hx) {
  const long long plane = (long long)rows * cols;
  float* p = im + blockIdx.y * plane;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < plane;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = int(t / cols), j = int(t - (long long)(t / cols) * cols);
    float s = 1.f;
    if (i < hy) s = __ldg(wy + i);
    else if (i > rows - 1 - hy) s = __ldg(wy + rows - 1 - i);
    if (j < hx) s *= __ldg(wx + j);
    else if (j > cols - 1 - hx) s *= __ldg(wx + cols - 1 - j);
    if (s != 1.f) p[t] *= s;
  }
}

cudaError_t launch_edgetaper(float* im, int rows, int cols, const float* wy, int hy, const float* wx,
                             int hx, int batch, cudaStream_t st) {
  const long long plane = (long long)rows * cols;
  const int blocks = (int)((plane + 255) / 256 < 1184 ? (plane + 255) / 256 : 1184);
  edgetaper_kernel<<<dim3(blocks, batch), 256, 0, st>>>(im, rows, cols, wy, hy, wx, hx);
  return cudaGetLastError();
}

}  // namespace eff
