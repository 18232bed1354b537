// EFF kernel instantiations for the 64x64 frame.
#include "eff_launch.cuh"

namespace eff {
cudaError_t launch_n64(int op, const Params& P, int K, int batch, int threads, size_t smem, cudaStream_t st) {
  return launch_n<64>(op, P, K, batch, threads, smem, st);
}
}  // namespace eff
