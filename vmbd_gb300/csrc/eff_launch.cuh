// Launch helpers shared by the per-frame-size translation units.
#pragma once
#include <atomic>
#include "eff_kernels.cuh"

namespace eff {

// Shared-memory bytes of one CTA: twiddles + frame + per-group exchange scratch.
inline size_t smem_bytes(int N, int op, const Params& P, int threads) {
  const int G = N / 16;
  const int scr = 16 * (G + 1) + 8;
  return sizeof(float2) * ((size_t)N + (size_t)frame_rows(P, op) * frame_pitch(N) +
                           (size_t)(threads / G) * scr);
}

template <int N, int OP>
cudaError_t launch_one(const Params& P, int K, int batch, int threads, size_t smem, cudaStream_t st) {
  static std::atomic<int> attr_bytes[64];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 64 || attr_bytes[dev].load() < (int)smem) {
    e = cudaFuncSetAttribute(eff_kernel<N, OP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (dev < 64) attr_bytes[dev].store((int)smem);
  }
  eff_kernel<N, OP><<<dim3(K, batch), threads, smem, st>>>(P);
  return cudaGetLastError();
}

template <int N>
cudaError_t launch_n(int op, const Params& P, int K, int batch, int threads, size_t smem, cudaStream_t st) {
  switch (op) {
    case OP_SPEC_IMAGE: return launch_one<N, OP_SPEC_IMAGE>(P, K, batch, threads, smem, st);
    case OP_SPEC_PSF: return launch_one<N, OP_SPEC_PSF>(P, K, batch, threads, smem, st);
    case OP_FWD_IMAGE: return launch_one<N, OP_FWD_IMAGE>(P, K, batch, threads, smem, st);
    case OP_FWD_PSF: return launch_one<N, OP_FWD_PSF>(P, K, batch, threads, smem, st);
    case OP_FWD_BOTH: return launch_one<N, OP_FWD_BOTH>(P, K, batch, threads, smem, st);
    case OP_ADJ: return launch_one<N, OP_ADJ>(P, K, batch, threads, smem, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_n64(int op, const Params& P, int K, int batch, int threads, size_t smem, cudaStream_t st);
cudaError_t launch_n128(int op, const Params& P, int K, int batch, int threads, size_t smem, cudaStream_t st);
cudaError_t launch_n256(int op, const Params& P, int K, int batch, int threads, size_t smem, cudaStream_t st);

}  // namespace eff
