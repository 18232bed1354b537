// Small fused kernels of the online multi-frame blind deconvolution step.
//
// PSF step: projected gradient with Barzilai-Borwein step sizes (the step
// rule of PBB, optGPU.py:222-226, alternating <dx,dx>/<dx,dg> and
// <dx,dg>/<dg,dg>) and the Euclidean simplex projection; the first step of
// a frame uses the exact line search <g,g>/||Xg||^2 of the quadratic.
// Image step: the multiplicative update of vmbd_chimney.py:143-147,
// x *= max(Ft(m y) / (Ft(m F x) + tol), tol), then x <= max over the
// interior of x.
#include <cuda_runtime.h>

namespace eff {

constexpr int kMfbdThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// out[0] += sum (a-ap)^2 over na, out[2] += sum (b-bp)^2 over nb,
// out[1] += sum (a-ap)(b-bp) over min(na, nb); ap / bp may be null.
__global__ void __launch_bounds__(kMfbdThreads) dots3_kernel(const float* a, const float* ap, long long na,
                                                             const float* b, const float* bp, long long nb,
                                                             double* out) {
  double s0 = 0, s1 = 0, s2 = 0;
  const long long n = na > nb ? na : nb;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float u = i < na ? a[i] - (ap ? ap[i] : 0.f) : 0.f;
    const float v = i < nb ? b[i] - (bp ? bp[i] : 0.f) : 0.f;
    s0 += double(u) * u;
    s1 += double(u) * v;
    s2 += double(v) * v;
  }
  s0 = warp_sum(s0);
  s1 = warp_sum(s1);
  s2 = warp_sum(s2);
  // one atomic per block and value (per-warp atomics on the same three
  // addresses serialise)
  __shared__ double part[3][kMfbdThreads / 32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    part[0][w] = s0;
    part[1][w] = s1;
    part[2][w] = s2;
  }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      double v = l < nw ? part[q][l] : 0.0;
      v = warp_sum(v);
      if (l == 0) atomicAdd(out + q, v);
    }
  }
}

// Deterministic block sum (float2), every thread gets the totals.
__device__ __forceinline__ float2 block_sum2f(float a, float b, float2* red) {
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

// Step size from the dot products.  mode 0: exact line search
// dots = (<g,g>, ., ||Xg||^2); mode 1/2: BB1/BB2 with dots = (<dx,dx>,
// <dx,dg>, <dg,dg>); a non-positive curvature keeps the previous step.
__device__ __forceinline__ float pg_step_size(const double* dots, int mode, float prev) {
  double s;
  if (mode == 0) s = dots[2] > 0 ? dots[0] / dots[2] : 0.0;
  else if (dots[1] <= 0) s = prev;
  else if (mode == 1) s = dots[0] / dots[1];
  else s = dots[2] > 0 ? dots[1] / dots[2] : prev;
  if (!(s > 0) || !isfinite(s)) s = prev;
  return (float)s;
}

// Side job of a kernel: zero [z, z + nz) (a buffer a later call accumulates
// into and that this kernel neither reads nor writes otherwise), grid-stride.
__device__ __forceinline__ void zero_side(float* z, long long nz) {
  if (!z) return;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nz; t += (long long)gridDim.x * blockDim.x)
    z[t] = 0.f;
}

// One PSF per CTA: fp <- f, gp <- g, f <- P_simplex(f - s g).  state[0] holds
// the step size (written by CTA 0).
__global__ void __launch_bounds__(kMfbdThreads) pg_step_kernel(float* f, const float* g, float* fp, float* gp,
                                                               int n, const double* dots, int mode,
                                                               float* state, float* zero_f, long long zero_n) {
  extern __shared__ float v[];
  __shared__ float2 red[32];
  zero_side(zero_f, zero_n);
  const float s = pg_step_size(dots, mode, state[0]);
  const long long base = (long long)blockIdx.x * n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const float fi = f[base + i], gi = g[base + i];
    fp[base + i] = fi;
    gp[base + i] = gi;
    v[i] = fi - s * gi;
  }
  __syncthreads();
  if (blockIdx.x == 0 && threadIdx.x == 0) state[0] = s;
  // Michelot's active-set iteration for the simplex projection.
  float sum = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) sum += v[i];
  float2 t = block_sum2f(sum, 0.f, red);
  float tau = (t.x - 1.f) / float(n);
  int count = n;
  for (int it = 0; it <= n; ++it) {
    float ss = 0.f, cc = 0.f;
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      if (v[i] > tau) {
        ss += v[i];
        cc += 1.f;
      }
    t = block_sum2f(ss, cc, red);
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
  for (int i = threadIdx.x; i < n; i += blockDim.x) f[base + i] = fmaxf(v[i] - tau, 0.f);
}

// Block maximum of a non-negative value, then one atomicMax on its bits
// (non-negative floats order like their bit patterns).
__device__ __forceinline__ void block_max_atomic(float m, unsigned* bits) {
  __shared__ float part[kMfbdThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) part[w] = m;
  __syncthreads();
  if (w == 0) {
    float v = l < (int)(blockDim.x >> 5) ? part[l] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (l == 0) atomicMax(bits, __float_as_uint(fmaxf(v, 0.f)));
  }
}

// out_bits <- max(0, max_i a[i]) as float bits (non-negative floats order
// like their bit patterns).
__global__ void __launch_bounds__(kMfbdThreads) max_nonneg_kernel(const float* a, long long n, unsigned* out_bits) {
  float m = 0.f;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x)
    m = fmaxf(m, a[t]);
  block_max_atomic(m, out_bits);
}

// x *= max(num / (den + tol), tol); xmax_bits <- max over the interior
// [b0, rows-b0) x [b1, cols-b1) of the updated x (x >= 0, so the float bit
// patterns order like the values).  num below floor * max(num) is taken as
// 0: where no data reaches a pixel, num and den are 0 in exact arithmetic
// (factor tol) but FP32 transform noise of ~1e-8 of the image scale, far
// above tol, and their ratio would be noise over noise.
__global__ void __launch_bounds__(kMfbdThreads) mu_update_kernel(float* x, const float* num, const float* den,
                                                                 float tol, int rows, int cols, int b0, int b1,
                                                                 const unsigned* num_max_bits, float floor_rel,
                                                                 unsigned* xmax_bits, float* zero_f, long long zero_n) {
  zero_side(zero_f, zero_n);
  const long long n = (long long)rows * cols;
  const float nfloor = floor_rel * __uint_as_float(*num_max_bits);
  float m = 0.f;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const float nu = num[t] > nfloor ? num[t] : 0.f;
    const float fac = fmaxf(nu / (den[t] + tol), tol);
    const float xv = x[t] * fac;
    x[t] = xv;
    const int i = int(t / cols), j = int(t % cols);
    if (i >= b0 && i < rows - b0 && j >= b1 && j < cols - b1) m = fmaxf(m, xv);
  }
  block_max_atomic(m, xmax_bits);
}

__global__ void __launch_bounds__(kMfbdThreads) clamp_max_kernel(float* x, long long n, const unsigned* xmax_bits) {
  const float mx = __uint_as_float(*xmax_bits);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x)
    x[t] = fminf(x[t], mx);
}

// Grid for n elements: at most 4 elements per thread before growing the
// grid, capped at 2 blocks per SM of a 152-SM part.
static int grid_for(long long n) {
  const long long b = (n + 4LL * kMfbdThreads - 1) / (4LL * kMfbdThreads);
  return (int)(b < 304 ? (b < 1 ? 1 : b) : 304);
}

cudaError_t launch_dots3(const float* a, const float* ap, long long na, const float* b, const float* bp,
                         long long nb, double* out, bool zeroed, cudaStream_t st) {
  if (!zeroed) {
    cudaError_t e = cudaMemsetAsync(out, 0, 3 * sizeof(double), st);
    if (e != cudaSuccess) return e;
  }
  dots3_kernel<<<grid_for(na > nb ? na : nb), kMfbdThreads, 0, st>>>(a, ap, na, b, bp, nb, out);
  return cudaGetLastError();
}

cudaError_t launch_pg_step(float* f, const float* g, float* fp, float* gp, int K, int n, const double* dots,
                           int mode, float* state, float* zero_f, long long zero_n, cudaStream_t st) {
  pg_step_kernel<<<K, kMfbdThreads, n * sizeof(float), st>>>(f, g, fp, gp, n, dots, mode, state, zero_f, zero_n);
  return cudaGetLastError();
}

cudaError_t launch_max_nonneg(const float* a, long long n, unsigned* out_bits, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(out_bits, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  max_nonneg_kernel<<<grid_for(n), kMfbdThreads, 0, st>>>(a, n, out_bits);
  return cudaGetLastError();
}

cudaError_t launch_mu_update(float* x, const float* num, const float* den, float tol, int rows, int cols,
                             int b0, int b1, const unsigned* num_max_bits, float floor_rel, unsigned* xmax_bits,
                             bool zeroed, float* zero_f, long long zero_n, cudaStream_t st) {
  cudaError_t e;
  if (!zeroed && (e = cudaMemsetAsync(xmax_bits, 0, sizeof(unsigned), st)) != cudaSuccess) return e;
  const long long n = (long long)rows * cols;
  mu_update_kernel<<<grid_for(n), kMfbdThreads, 0, st>>>(x, num, den, tol, rows, cols, b0, b1, num_max_bits,
                                                          floor_rel, xmax_bits, zero_f, zero_n);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  clamp_max_kernel<<<grid_for(n), kMfbdThreads, 0, st>>>(x, n, xmax_bits);
  return cudaGetLastError();
}

}  // namespace eff
