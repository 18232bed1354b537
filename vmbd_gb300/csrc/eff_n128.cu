// EFF kernel instantiations for the 128x128 frame.
#include "eff_launch.cuh"

namespace eff {
cudaError_t launch_n128(int op, const Params& P, int K, int batch, int threads, size_t smem, cudaStream_t st) {
  return launch_n<128>(op, P, K, batch, threads, smem, st);
}
}  // namespace eff
