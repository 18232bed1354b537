// EFF kernel instantiations for the 256x256 frame (single CTA and 2-CTA cluster per patch).
#include "eff_launch.cuh"

namespace eff {
cudaError_t launch_n256(int op, int CL, const Params& P, int K, int batch, int threads, size_t smem, cudaStream_t st,
                        const CUtensorMap* xmap) {
  return launch_n<256>(op, CL, P, K, batch, threads, smem, st, xmap);
}
}  // namespace eff
