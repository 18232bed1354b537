// Deterministic overlap-add gather (eff_ola.cu).
#pragma once
#include <cuda_runtime.h>

namespace eff {

struct GatherArgs {
  const float* tiles;  // [csf0 * csf1][th][tw], patch k = m * csf1 + n
  int th, tw;          // tile rows / columns
  int csf0, csf1, hop0, hop1;
  int off0, off1;      // output pixel (i, j) lies at (i + off0 - m hop0, j + off1 - n hop1) of tile (m, n)
  int rows, cols;      // output size (0 x 0: only the loss)
  const float* sub;    // nullable: subtracted from every output pixel
  float* out;
  const double* loss_part;  // nullable: per-CTA loss shares, summed in order into *loss
  int nparts;
  double* loss;
};

cudaError_t launch_ola_gather(const GatherArgs& A, int num_sms, cudaStream_t st);

}  // namespace eff
