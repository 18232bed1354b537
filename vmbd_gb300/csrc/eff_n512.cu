// Launches for the 512x512 frame (32 values per lane, 16 lanes per
// transform) on clusters of 4 CTAs, or of 8 for extents whose quarter frame
// does not fit.  The kernels themselves are instantiated in eff_n512_k*.cu,
// a few per translation unit, so that they compile in parallel.
#include "eff_launch.cuh"

namespace eff {
#define EFF_N512_EXTERN(OP, CL) \
  extern template cudaError_t launch_one<512, OP, CL>(const Params&, int, int, int, size_t, cudaStream_t, \
                                                     const CUtensorMap*);
EFF_N512_EXTERN(0, 4) EFF_N512_EXTERN(1, 4) EFF_N512_EXTERN(2, 4) EFF_N512_EXTERN(3, 4)
EFF_N512_EXTERN(4, 4) EFF_N512_EXTERN(5, 4) EFF_N512_EXTERN(6, 4)
EFF_N512_EXTERN(0, 8) EFF_N512_EXTERN(1, 8) EFF_N512_EXTERN(2, 8) EFF_N512_EXTERN(3, 8)
EFF_N512_EXTERN(4, 8) EFF_N512_EXTERN(5, 8) EFF_N512_EXTERN(6, 8)
#undef EFF_N512_EXTERN

cudaError_t launch_n512(int op, int CL, const Params& P, int K, int batch, int threads, size_t smem, cudaStream_t st,
                        const CUtensorMap* xmap) {
  if (CL == 4) return launch_ncl<512, 4>(op, P, K, batch, threads, smem, st, xmap);
  if (CL == 8) return launch_ncl<512, 8>(op, P, K, batch, threads, smem, st, xmap);
  return cudaErrorInvalidValue;
}
}  // namespace eff
