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

// Up to two byte ranges to clear (4-byte aligned, sizes multiples of 4;
// nullptr / 0 for an unused range).
struct ZeroArgs {
  void* p[2];
  long long bytes[2];
};

// Clears the ranges with a kernel whose blocks let the next kernel on the
// stream start at once, when that one is launched with programmatic stream
// serialization; that kernel waits (griddepcontrol.wait) before its first
// access to the ranges, so the clear overlaps its start.
cudaError_t launch_zero(const ZeroArgs& Z, int num_sms, cudaStream_t st);

}  // namespace eff
