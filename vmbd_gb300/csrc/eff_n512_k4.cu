// Frame-512 kernels on 8-CTA clusters, ops 0 1 2 (see eff_n512.cu).
#include "eff_launch.cuh"

namespace eff {
template cudaError_t launch_one<512, 0, 8>(const Params&, int, int, int, size_t, cudaStream_t, const CUtensorMap*);
template cudaError_t launch_one<512, 1, 8>(const Params&, int, int, int, size_t, cudaStream_t, const CUtensorMap*);
template cudaError_t launch_one<512, 2, 8>(const Params&, int, int, int, size_t, cudaStream_t, const CUtensorMap*);
}  // namespace eff
