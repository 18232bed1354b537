// Frame-512 kernels on 4-CTA clusters, ops 5 6 (see eff_n512.cu).
#include "eff_launch.cuh"

namespace eff {
template cudaError_t launch_one<512, 5, 4>(const Params&, int, int, int, size_t, cudaStream_t, const CUtensorMap*);
template cudaError_t launch_one<512, 6, 4>(const Params&, int, int, int, size_t, cudaStream_t, const CUtensorMap*);
}  // namespace eff
