// EFF kernel instantiations for the 256x256 frame.
#include "eff_launch.cuh"

namespace eff {
cudaError_t launch_n256(int op, const Params& P, int K, int batch, int threads, size_t smem, cudaStream_t st) {
  return launch_n<256>(op, P, K, batch, threads, smem, st);
}
}  // namespace eff
