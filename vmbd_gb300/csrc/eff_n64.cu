// EFF kernel instantiations for the 64x64 frame (single CTA and 2-CTA cluster per patch).
#include "eff_launch.cuh"

namespace eff {
cudaError_t launch_n64(int op, int CL, const Params& P, int K, int batch, int threads, size_t smem, cudaStream_t st,
                        const CUtensorMap* xmap) {
  return launch_n<64>(op, CL, P, K, batch, threads, smem, st, xmap);
}
}  // namespace eff
