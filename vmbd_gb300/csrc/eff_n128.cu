// EFF kernel instantiations for the 128x128 frame (single CTA and 2-CTA cluster per patch).
#include "eff_launch.cuh"

namespace eff {
cudaError_t launch_n128(int op, int CL, const Params& P, int K, int batch, int threads, size_t smem, cudaStream_t st,
                        const CUtensorMap* xmap) {
  return launch_n<128>(op, CL, P, K, batch, threads, smem, st, xmap);
}
}  // namespace eff
