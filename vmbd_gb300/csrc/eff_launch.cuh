// Launch helpers shared by the per-frame-size translation units.
#pragma once
#include <atomic>
#include <cstring>
#include "eff_kernels.cuh"

namespace eff {

// Shared-memory bytes of one CTA: twiddles + frame (its share of the columns)
// + per-group exchange scratch + the DC unit's stash (2N) + the row-owned
// output block and its mbarrier (frame-128 pairs); with staged
// spectra (P.stage_spec) also an alignment slot, the staged columns and the
// mbarrier; with an image tile (P.tile_rows) the tile, its alignment and its
// mbarrier.
inline size_t smem_bytes(int N, int op, const Params& P, int threads, int CL) {
  const int R = lane_values(N), G = N / R;
  const int scr = group_scratch(N);
  size_t n = (size_t)N + (size_t)frame_rows(P, op) * frame_pitch(N, CL) + (size_t)(threads / G) * scr +
             2 * (size_t)N + (size_t)out_rows_f2(P, op, N, CL);
  if (const int nst = staged_specs(P, op)) n += 1 + (size_t)nst * staged_cols(N, CL) * (N + kSpecPad) + 1;
  n += (size_t)image_tile_f2(P, op);
  return sizeof(float2) * n;
}

template <int N, int OP, int CL>
cudaError_t launch_one(const Params& P, int K, int batch, int threads, size_t smem, cudaStream_t st,
                       const CUtensorMap* xmap) {
  static std::atomic<int> attr_bytes[64];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  auto kern = eff_kernel<N, OP, CL>;
  // an error status an earlier runtime call left behind (already returned to
  // its caller) must not be read back as this launch's result below
  (void)cudaGetLastError();
  if (dev >= 64 || attr_bytes[dev].load() < (int)smem) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (dev < 64) attr_bytes[dev].store((int)smem);
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(K * CL, batch);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[2];
  int na = 0;
  if (CL > 1) {
    attr[na].id = cudaLaunchAttributeClusterDimension;
    attr[na].val.clusterDim.x = CL;
    attr[na].val.clusterDim.y = 1;
    attr[na].val.clusterDim.z = 1;
    ++na;
  }
  if (P.pdl) {  // may start while its predecessor on the stream runs; waits before reading
    attr[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[na].val.programmaticStreamSerializationAllowed = 1;
    ++na;
  }
  cfg.attrs = attr;
  cfg.numAttrs = na;
  // the image's tensor map (P.tile_rows > 0), else an unused placeholder
  CUtensorMap none;
  std::memset(&none, 0, sizeof(none));
  e = cudaLaunchKernelEx(&cfg, kern, P, xmap && P.tile_rows > 0 ? *xmap : none);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

template <int N, int CL>
cudaError_t launch_ncl(int op, const Params& P, int K, int batch, int threads, size_t smem, cudaStream_t st,
                       const CUtensorMap* xmap) {
  switch (op) {
    case OP_SPEC_IMAGE: return launch_one<N, OP_SPEC_IMAGE, CL>(P, K, batch, threads, smem, st, xmap);
    case OP_SPEC_PSF: return launch_one<N, OP_SPEC_PSF, CL>(P, K, batch, threads, smem, st, xmap);
    case OP_FWD_IMAGE: return launch_one<N, OP_FWD_IMAGE, CL>(P, K, batch, threads, smem, st, xmap);
    case OP_FWD_PSF: return launch_one<N, OP_FWD_PSF, CL>(P, K, batch, threads, smem, st, xmap);
    case OP_FWD_BOTH: return launch_one<N, OP_FWD_BOTH, CL>(P, K, batch, threads, smem, st, xmap);
    case OP_ADJ: return launch_one<N, OP_ADJ, CL>(P, K, batch, threads, smem, st, xmap);
    case OP_DECONV: return launch_one<N, OP_DECONV, CL>(P, K, batch, threads, smem, st, xmap);
    default: return cudaErrorInvalidValue;
  }
}

template <int N>
cudaError_t launch_n(int op, int CL, const Params& P, int K, int batch, int threads, size_t smem,
                     cudaStream_t st, const CUtensorMap* xmap) {
  if (CL != 1 && CL != 2) return cudaErrorInvalidValue;
  return CL == 2 ? launch_ncl<N, 2>(op, P, K, batch, threads, smem, st, xmap)
                 : launch_ncl<N, 1>(op, P, K, batch, threads, smem, st, xmap);
}

cudaError_t launch_n64(int op, int CL, const Params& P, int K, int batch, int threads, size_t smem, cudaStream_t st,
                        const CUtensorMap* xmap = nullptr);
cudaError_t launch_n128(int op, int CL, const Params& P, int K, int batch, int threads, size_t smem, cudaStream_t st,
                        const CUtensorMap* xmap = nullptr);
cudaError_t launch_n192(int op, int CL, const Params& P, int K, int batch, int threads, size_t smem, cudaStream_t st,
                        const CUtensorMap* xmap = nullptr);
cudaError_t launch_n256(int op, int CL, const Params& P, int K, int batch, int threads, size_t smem, cudaStream_t st,
                        const CUtensorMap* xmap = nullptr);
// frame 512: CL = 4 or 8 only
cudaError_t launch_n512(int op, int CL, const Params& P, int K, int batch, int threads, size_t smem, cudaStream_t st,
                        const CUtensorMap* xmap = nullptr);

}  // namespace eff
