// EFF kernel instantiations for the 192x192 frame (24 x 8 mixed radix) (single CTA and 2-CTA cluster per patch).
#include "eff_launch.cuh"

namespace eff {
cudaError_t launch_n192(int op, int CL, const Params& P, int K, int batch, int threads, size_t smem, cudaStream_t st,
                        const CUtensorMap* xmap) {
  return launch_n<192>(op, CL, P, K, batch, threads, smem, st, xmap);
}
}  // namespace eff
