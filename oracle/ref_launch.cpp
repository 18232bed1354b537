// CPU execution of the reference's hot-path CUDA kernels (gputools.cu).
//
// TEST INFRASTRUCTURE ONLY (oracle).  The reference source is compiled from
// where it lies: the build recipe (oracle/build_ref.py) passes its path as
// REF_GPUTOOLS_CU and this file #includes it after a shim that maps the CUDA
// execution model onto plain C++ (thread-local blockIdx/threadIdx set by a
// serial loop over the launch grid).  The included kernels use no shared
// memory and no barriers, so a serial loop reproduces them exactly.
//
// Each ref_* entry point takes the grid and block sizes the reference's
// Python wrapper (gputools.py) computes, followed by the kernel's own
// arguments, and runs the launch.

#include <cstdint>
#include <cstddef>

struct ShimDim3 {
  unsigned x, y, z;
};
static thread_local ShimDim3 blockIdx, threadIdx, blockDim, gridDim;

#define __global__ static
#define __device__ static
#define __constant__ static

static inline unsigned __umul24(unsigned a, unsigned b) {
  return (a & 0xffffffu) * (b & 0xffffffu);
}
// CUDA's integer min(): mixed signed/unsigned arguments compare as unsigned.
template <class A, class B>
static inline auto min(A a, B b) -> decltype(a + b) {
  typedef decltype(a + b) T;
  return (T(a) < T(b)) ? T(a) : T(b);
}

#include REF_GPUTOOLS_CU

template <class F>
static void run_grid(unsigned gx, unsigned gy, unsigned bx, unsigned by, F f) {
  gridDim = {gx, gy, 1};
  blockDim = {bx, by, 1};
  for (unsigned y = 0; y < gy; ++y)
    for (unsigned x = 0; x < gx; ++x)
      for (unsigned ty = 0; ty < by; ++ty)
        for (unsigned tx = 0; tx < bx; ++tx) {
          blockIdx = {x, y, 0};
          threadIdx = {tx, ty, 0};
          f();
        }
}

#define G unsigned gx, unsigned gy, unsigned bx, unsigned by
#define RUN(call) run_grid(gx, gy, bx, by, [&] { call; })

extern "C" {

void ref_zeroPadKernel(G, float* dx, int m, int n, float* dy, int p, int q, int s, int t) {
  RUN(zeroPadKernel(dx, m, n, dy, p, q, s, t));
}

void ref_zeroPadComplexKernel(G, cufftComplex* dx, int m, int n, float* dy, int p, int q, int s, int t) {
  RUN(zeroPadComplexKernel(dx, m, n, dy, p, q, s, t));
}

void ref_chop_pad_Kernel(G, float* dx, int xm, int xn, int xr, float* dy, int ym, int yn, int wm,
                         int wn, int om, int on, int cm, int cn, int hopm, int hopn) {
  RUN(chop_pad_Kernel(dx, xm, xn, xr, dy, ym, yn, wm, wn, om, on, cm, cn, hopm, hopn));
}

void ref_chop_pad_ComplexKernel(G, cufftComplex* dx, int xm, int xn, int xr, float* dy, int ym,
                                int yn, int wm, int wn, int om, int on, int cm, int cn, int hopm,
                                int hopn) {
  RUN(chop_pad_ComplexKernel(dx, xm, xn, xr, dy, ym, yn, wm, wn, om, on, cm, cn, hopm, hopn));
}

void ref_chop_mod_pad_ComplexKernel(G, cufftComplex* dx, int xm, int xn, int xr, float* dy, int ym,
                                    int yn, float* dw, int wm, int wn, int om, int on, int cm,
                                    int cn, int hopm, int hopn) {
  RUN(chop_mod_pad_ComplexKernel(dx, xm, xn, xr, dy, ym, yn, dw, wm, wn, om, on, cm, cn, hopm,
                                 hopn));
}

void ref_pad_stack_ComplexKernel(G, float* dx, int xk, int xm, int xn, cufftComplex* dxp, int pm,
                                 int pn, int om, int on) {
  RUN(pad_stack_ComplexKernel(dx, xk, xm, xn, dxp, pm, pn, om, on));
}

void ref_crop_stack_Kernel(G, float* dx, int xk, int xm, int xn, float* dxp, int pm, int pn, int om,
                           int on) {
  RUN(crop_stack_Kernel(dx, xk, xm, xn, dxp, pm, pn, om, on));
}

void ref_crop_Kernel(G, float* dx, int m, int n, float* dy, int p, int q, int s, int t) {
  RUN(crop_Kernel(dx, m, n, dy, p, q, s, t));
}

void ref_ola_Kernel_test(G, float* out, float* in, unsigned outm, unsigned outn, unsigned inm,
                         unsigned inn, unsigned wm, unsigned wn, unsigned om, unsigned on,
                         unsigned cm, unsigned cn, unsigned hopm, unsigned hopn) {
  RUN(ola_Kernel_test(out, in, outm, outn, inm, inn, wm, wn, om, on, cm, cn, hopm, hopn));
}

void ref_ola_ComplexKernel_test(G, float* out, cufftComplex* in, unsigned outm, unsigned outn,
                                unsigned inm, unsigned inn, unsigned wm, unsigned wn, unsigned om,
                                unsigned on, unsigned cm, unsigned cn, unsigned hopm,
                                unsigned hopn) {
  RUN(ola_ComplexKernel_test(out, in, outm, outn, inm, inn, wm, wn, om, on, cm, cn, hopm, hopn));
}

void ref_comp_ola_deconv_Kernel(G, cufftComplex* out, int outk, int outm, int outn, cufftComplex* f,
                                cufftComplex* y, cufftComplex* L, float alpha, float beta) {
  RUN(comp_ola_deconv_Kernel(out, outk, outm, outn, f, y, L, alpha, beta));
}

}  // extern "C"
