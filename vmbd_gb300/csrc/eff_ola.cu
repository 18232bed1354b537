// Deterministic overlap-add: the gather half.
//
// A plan created with EFF_GEOM_DETERMINISTIC has its kernels store every
// patch's output tile (forward: the E0 x E1 full-convolution tile; image
// adjoint / deconvolution: the sw0 x sw1 tile) instead of adding it into the
// image with atomics.  This kernel then forms each output pixel as the sum of
// the tiles that cover it, always in the same order (patch rows ascending,
// then patch columns), so repeated calls give bit-identical results -- the
// reference's overlap-add is such a gather too (ola_Kernel_test,
// gputools.cu:276-314: one thread per output pixel over the covering
// patches).  It also subtracts the observation of a residual forward and sums
// the adjoint's per-CTA loss shares in CTA order.
#include <cuda_runtime.h>

#include "eff_ola.h"

namespace eff {

__global__ void __launch_bounds__(256) ola_gather_kernel(GatherArgs A) {
  // launched with programmatic stream serialization: the kernel after it may
  // be scheduled now, and this one waits for the kernel storing the tiles
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const long long n = (long long)A.rows * A.cols;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(p / A.cols), j = (int)(p - (long long)(p / A.cols) * A.cols);
    const int gi = i + A.off0, gj = j + A.off1;  // position in patch-origin coordinates
    // patches m with m hop0 <= gi < m hop0 + th (and likewise n)
    const int di = gi - A.th, dj = gj - A.tw;
    const int m_lo = di < 0 ? 0 : di / A.hop0 + 1, m_hi = min(A.csf0 - 1, gi / A.hop0);
    const int n_lo = dj < 0 ? 0 : dj / A.hop1 + 1, n_hi = min(A.csf1 - 1, gj / A.hop1);
    float acc = 0.f;
    for (int m = m_lo; m <= m_hi; ++m) {
      const float* row = A.tiles + ((long long)m * A.csf1) * A.th * A.tw + (long long)(gi - m * A.hop0) * A.tw;
      for (int nn = n_lo; nn <= n_hi; ++nn)
        acc += __ldg(row + (long long)nn * A.th * A.tw + (gj - nn * A.hop1));
    }
    if (A.sub) acc -= __ldg(A.sub + p);
    A.out[p] = acc;
  }
  if (A.loss && blockIdx.x == 0 && threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < A.nparts; ++q) t += A.loss_part[q];
    *A.loss = t;
  }
}

cudaError_t launch_ola_gather(const GatherArgs& A, int num_sms, cudaStream_t st) {
  const long long n = (long long)A.rows * A.cols;
  long long blocks = (n + 255) / 256;
  const long long cap = 8LL * (num_sms > 0 ? num_sms : 1);
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)blocks);
  cfg.blockDim = dim3(256);
  cfg.stream = st;
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr.val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  cudaError_t e = cudaLaunchKernelEx(&cfg, ola_gather_kernel, A);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

// Clear of an output that the next kernel accumulates into.  Each block
// triggers the dependent launch first: the clear then runs beside that
// kernel's transforms, which only need the output at their end.
__global__ void __launch_bounds__(256) zero_kernel(ZeroArgs Z) {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long nt = (long long)gridDim.x * blockDim.x;
#pragma unroll 1
  for (int r = 0; r < 2; ++r) {
    char* p = static_cast<char*>(Z.p[r]);
    const long long n = Z.bytes[r];
    if (!p || n <= 0) continue;
    // 4-byte words up to the first 16-byte boundary, 16-byte stores, then words
    long long head = (long long)((16 - (reinterpret_cast<unsigned long long>(p) & 15ull)) & 15ull);
    if (head > n) head = n;
    const long long n16 = (n - head) >> 4;
    const long long tail0 = head + (n16 << 4);
    if (t0 < head / 4) reinterpret_cast<unsigned*>(p)[t0] = 0u;
    uint4* q = reinterpret_cast<uint4*>(p + head);
    for (long long i = t0; i < n16; i += nt) q[i] = make_uint4(0u, 0u, 0u, 0u);
    const long long ntail = (n - tail0) / 4;
    if (t0 < ntail) reinterpret_cast<unsigned*>(p + tail0)[t0] = 0u;
  }
}

cudaError_t launch_zero(const ZeroArgs& Z, int num_sms, cudaStream_t st) {
  long long n16 = 0;
  for (int r = 0; r < 2; ++r) {
    if (Z.p[r] && ((reinterpret_cast<unsigned long long>(Z.p[r]) & 3ull) || (Z.bytes[r] & 3)))
      return cudaErrorInvalidValue;
    if (Z.p[r] && Z.bytes[r] > 0) n16 = n16 > Z.bytes[r] / 16 ? n16 : Z.bytes[r] / 16;
  }
  long long blocks = (n16 + 255) / 256;
  const long long cap = num_sms > 0 ? num_sms : 1;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  zero_kernel<<<(unsigned)blocks, 256, 0, st>>>(Z);
  return cudaGetLastError();
}

}  // namespace eff
