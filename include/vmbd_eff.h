/* vmbd_eff.h -- C ABI of the GB300 efficient-filter-flow (EFF) operator.
 *
 * Drop-in for the device work behind VMBD's OlaGPU class (olaGPU.py) and its
 * gputools wrappers.  All data pointers are caller-owned DEVICE pointers
 * (float32, C order); `stream` is a cudaStream_t passed as void* (NULL = the
 * legacy default stream).  Every entry point returns an EFF_* status and
 * never aborts; eff_last_error() describes the last failure on the calling
 * thread.  Plans are immutable after creation and may be used from several
 * host threads / streams at once.  A plan belongs to the device that was
 * current at its creation: a call made while another device is current
 * returns EFF_ERR_INVALID before it queues any work.  The compute entry
 * points allocate nothing.
 *
 * Geometry (per dim d): image sx, PSF sf, patch grid csf, patch size sw,
 * hop; K = csf0*csf1 patches, patch k = m*csf1 + n at (m*hop0, n*hop1);
 * E = sw + sf - 1; output size sy = sx-sf+1 (valid), sx (same), sx+sf-1
 * (full).
 *
 * Window stack (win2winaux, imagetools.py:398-454): the partition of unity
 * ws = w / chop(ola(w)) of a separable window w floored at 1e-16 is passed as
 * two per-dim tables of float pairs, win0 [csf0][sw0][2] and
 * win1 [csf1][sw1][2], entry (alpha, gamma) for patch row m (column n) and
 * local row r (column c) with global coordinate i = m*hop + r:
 *   alpha = a[r] / sum over covering patches m' of a[i - m'*hop]
 *           (a = the 1-D window scaled to max 1), or -1 when every covering
 *           patch has a zero window sample at i (the outermost rows);
 *   gamma = 1 / (number of patches covering i).
 * ws[k][r][c] = alpha0*alpha1 when both alphas are >= 0, else gamma0*gamma1.
 *
 * Batched calls run `batch` images of the same geometry, stored back to
 * back (image stride = the per-image size of each array).
 */
#ifndef VMBD_EFF_H
#define VMBD_EFF_H

#include <stddef.h>

/* The library is built with hidden symbol visibility; only these entry
 * points are exported. */
#if defined(__GNUC__)
#define EFF_API __attribute__((visibility("default")))
#else
#define EFF_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define EFF_OK 0
#define EFF_ERR_INVALID 1     /* bad argument: null pointer, inconsistent geometry */
#define EFF_ERR_UNSUPPORTED 2 /* geometry outside what the kernels handle */
#define EFF_ERR_CUDA 3        /* a CUDA runtime call failed */

#define EFF_MODE_VALID 0
#define EFF_MODE_SAME 1
#define EFF_MODE_FULL 2

#define EFF_OUT_ZEROED 1 /* flags: the call's accumulated output is already zero (no clear) */
#define EFF_LOSS_OF_Y 2  /* eff_adjoint_ex flags: y is already a residual; loss += 0.5 * sum y^2 */
#define EFF_AFTER_FORWARD 4 /* eff_adjoint_ex flags: the call directly follows, on the same stream,
                               the forward call that produced its inputs; its kernel may be
                               scheduled while that one runs and waits for it on the device */

#define EFF_OPERAND_IMAGE 0 /* eff_forward_ex: u is the image, spec the PSF spectrum */
#define EFF_OPERAND_PSF 1   /* eff_forward_ex: u is the PSF stack, spec the image spectrum */

#define EFF_ADJ_EXACT 0     /* exact transpose of the forward operator */
#define EFF_ADJ_REFERENCE 1 /* OlaGPU.cnvtp's truncated chop (olaGPU.py:276-286) */

typedef struct EffGeom {
  int sx[2];   /* image size */
  int sf[2];   /* PSF size */
  int csf[2];  /* patch grid */
  int sw[2];   /* patch size */
  int hop[2];  /* patch hop */
  int sfft;    /* FFT frame edge, 64, 128, 192, 256 or 512 (>= max(E)); 0 = the smallest power of two >= max(E) */
  int mode;    /* EFF_MODE_* */
  int threads; /* CTA size, a multiple of 32 up to the frame's maximum (512 for frame 64,
                  544 for 128, 384 for 192, 576 for 256, 256 for 512); 0 = the largest that
                  fits.  Lowered to fit shared memory. */
  int flags;   /* EFF_GEOM_* */
} EffGeom;

/* EffGeom.flags: deterministic overlap-add.  The kernels store each patch's
 * output tile and a gather kernel sums the tiles covering each pixel in a
 * fixed order (patch rows, then patch columns), as the reference's
 * ola_Kernel_test does (gputools.cu:276-314); the loss is summed in a fixed
 * order too.  Repeated calls give bit-identical outputs.  The plan then owns
 * a device scratch of one image's tiles (K * max(E0 E1, sw0 sw1) floats):
 * calls on several streams at once race on it, and batched calls run image
 * by image.  Costs one extra kernel per overlap-added output.  Not accepted
 * by eff_batch_create. */
#define EFF_GEOM_DETERMINISTIC 1

typedef struct EffPlan EffPlan;

/* Replaces OlaGPU.__init__'s geometry checks (olaGPU.py:95-168) and the
 * window upload of win2winaux (imagetools.py:437-454).  win0 [csf0*sw0*2] and
 * win1 [csf1*sw1*2] are HOST arrays; the plan keeps device copies. */
EFF_API int eff_plan_create(const EffGeom* geom, const float* win0, const float* win1, EffPlan** plan);
EFF_API int eff_plan_destroy(EffPlan* plan);

/* FFT frame edge chosen by the plan, and the bytes of one image's cached
 * spectrum (K * (N/2+1) * N complex64). */
EFF_API int eff_plan_frame(const EffPlan* plan, int* n);
EFF_API size_t eff_spectrum_bytes(const EffPlan* plan);

/* PSF spectrum cache of an F object: pad_stack_GPU + FFT, olaGPU.py:142-157.
 * f [batch, K, sf0, sf1] -> fhat [batch, spectrum]. */
EFF_API int eff_psf_spectrum(const EffPlan* plan, const float* f, void* fhat, int batch, void* stream);

/* Windowed-patch spectrum cache of an X object: chop_mod_pad_GPU + FFT,
 * olaGPU.py:147-157.  x [batch, sx0, sx1] -> xhat. */
EFF_API int eff_image_spectrum(const EffPlan* plan, const float* x, void* xhat, int batch, void* stream);

/* F.cnv(x), olaGPU.py:170-257: y = crop(OLA(IFFT(fhat * FFT(ws * chop(x))))).
 * y [batch, sy0, sy1] is overwritten.  xhat_out (nullable) receives the
 * windowed-patch spectrum of x as eff_image_spectrum would. */
EFF_API int eff_forward_image(const EffPlan* plan, const float* x, const void* fhat, float* y,
                      void* xhat_out, int batch, void* stream);

/* X.cnv(f), olaGPU.py:170-257 with the X object: same operator, the PSFs
 * transformed in-kernel.  fhat_out (nullable) receives f's spectrum. */
EFF_API int eff_forward_psf(const EffPlan* plan, const float* f, const void* xhat, float* y,
                    void* fhat_out, int batch, void* stream);

/* F.cnvtp(y) and X.cnvtp(y), olaGPU.py:261-311, sharing one transform of y.
 * gx [batch, sx0, sx1] (needs fhat) and/or gf [batch, K, sf0, sf1] (needs
 * xhat) are overwritten; pass NULL for an output that is not wanted.
 * adj_mode: EFF_ADJ_EXACT or EFF_ADJ_REFERENCE. */
EFF_API int eff_adjoint(const EffPlan* plan, const float* y, const void* fhat, const void* xhat, float* gx,
                float* gf, int adj_mode, int batch, void* stream);

/* y = EFF(x, f) from the raw image and PSFs in one kernel (the forward of an
 * autograd step): both operands are transformed in-kernel.  xhat_out /
 * fhat_out (nullable) receive the two spectra for a later eff_adjoint. */
EFF_API int eff_forward_both(const EffPlan* plan, const float* x, const float* f, float* y, void* xhat_out,
                     void* fhat_out, int batch, void* stream);

/* eff_adjoint of the residual r = y - y_obs (both [batch, sy0, sy1]) without
 * forming r; loss (nullable, double [batch]) receives 0.5 * ||y - y_obs||^2.
 * The gradient of that loss w.r.t. x and f (cnvinv_objfun/gradfun without
 * regularisation, olaGPU.py:756-811). */
EFF_API int eff_adjoint_residual(const EffPlan* plan, const float* y, const float* y_obs, const void* fhat,
                         const void* xhat, float* gx, float* gf, double* loss, int adj_mode,
                         int batch, void* stream);

/* r = EFF(x, f) - y_obs and both spectra (optional) in one kernel:
 * eff_forward_both whose CTAs also subtract a share each of the observation
 * (the additions commute with the overlap-add).  An adjoint of r with
 * EFF_LOSS_OF_Y then reads one plane instead of y and y_obs; eff_loss_grad
 * is these two kernels.  r must not alias y_obs. */
EFF_API int eff_forward_residual(const EffPlan* plan, const float* x, const float* f, const float* y_obs, float* r,
                         void* xhat_out, void* fhat_out, int batch, void* stream);

/* One loss/gradient step of 0.5 * ||EFF(x, f) - y_obs||^2: eff_forward_residual
 * then eff_adjoint_ex with EFF_LOSS_OF_Y (exact adjoints), with the residual and
 * the two spectra in a caller-provided device workspace of at least
 * eff_loss_grad_workspace_bytes(plan, batch) bytes.  gx or gf may be NULL
 * (not both); loss may be NULL. */
EFF_API size_t eff_loss_grad_workspace_bytes(const EffPlan* plan, int batch);
EFF_API int eff_loss_grad(const EffPlan* plan, const float* x, const float* f, const float* y_obs,
                  double* loss, float* gx, float* gf, void* workspace, size_t workspace_bytes,
                  int batch, void* stream);

/* eff_loss_grad without a workspace argument.  No counterpart in the
 * reference.  For callers that can neither allocate device memory nor pass a
 * workspace: an objective/gradient callback whose signature carries only the
 * data and the outputs, or a host program that reserves all device memory up
 * front or cannot afford cudaMalloc's implicit synchronisation.
 *
 * The scratch is a static device array of eff_static_scratch_bytes() bytes
 * (16 MiB) that every GPU loading the library keeps until the process exits;
 * larger geometries / batches return EFF_ERR_UNSUPPORTED.  The first call on
 * a device looks up the array's device address (cudaGetSymbolAddress) and
 * keeps it: make that first call before any stream capture, and do not call
 * it again on a device after cudaDeviceReset of that device (the address may
 * change).  All calls share the array; calls whose GPU work overlaps (other
 * streams or threads) race on it.  Allocates nothing. */
EFF_API size_t eff_static_scratch_bytes(void);
EFF_API int eff_loss_grad_static(const EffPlan* plan, const float* x, const float* f, const float* y_obs,
                         double* loss, float* gx, float* gf, int batch, void* stream);

/* PSF projections on [K, n] stacks (n = sf0*sf1), in place.
 * EFF_PROJ_CLIP_NORMALIZE: f = max(f, 0) then f /= sum(f) when sum > 1e-6
 *   (L-BFGS-B bounds olaGPU.py:404-411 + normalize gputools.py:1025-1044).
 * EFF_PROJ_SIMPLEX: Euclidean projection onto {f >= 0, sum f = 1}. */
#define EFF_PROJ_CLIP_NORMALIZE 0
#define EFF_PROJ_SIMPLEX 1
EFF_API int eff_project_psf(float* f, int K, int n, int proj_mode, void* stream);

/* projection.cu:3-27 as intended: w[b] = <fs, basis[b]> for b < nb, with
 * fs [n] and basis [nb, n]. */
EFF_API int eff_basis_project(const float* fs, const float* basis, float* w, int nb, int n, void* stream);

/* edgetaper_gpu (gputools.py:643-673, edgetaper.cu:6-31), in place on
 * [batch, rows, cols]: row i < hy is scaled by wy[i], row i > rows-1-hy by
 * wy[rows-1-i]; columns likewise with wx.  wy [hy], wx [hx] are DEVICE
 * tables (the first floor(sf/2) samples of the Bartlett-Hann window over
 * the product of the two windows' maxima, sf made odd). */
EFF_API int eff_edgetaper(float* im, int rows, int cols, const float* wy, int hy, const float* wx, int hx,
                  int batch, void* stream);

/* Fourier-division deconvolution, OlaGPU.deconv(y, mode='xdirect'),
 * olaGPU.py:550-609 with comp_ola_deconv_Kernel gputools.cu:316-341.  Per
 * patch k: the chop of y [batch, sy0, sy1] placed at frame offset off
 * (sf-1 valid, floor(sf/2) same) times the window at the frame origin, its
 * FFT Y, Z = conj(S) Y / (|S|^2 + alpha L + beta) with
 * L = |FFT([-1 1])|^2 + |FFT([-1; 1])|^2 over the plan's N x N frame, the
 * inverse FFT z; then
 *   u  [batch, sx0, sx1] (S = fhat, F object): overlap-add of the sw x sw
 *      crops of z (no window), cropped to sx;
 *   fz [batch, K, sf0, sf1] (S = xhat, X object): the sf x sf crops of z.
 * Either output may be NULL (not both); both are overwritten.  The division
 * happens in the plan's frame, so results equal the reference's when the
 * plan's N is the reference's frame (the power of two >= sw + sf - 1 in
 * both dims).  EFF_ERR_UNSUPPORTED for mode full (olaGPU.py:570-571). */
EFF_API int eff_deconv_xdirect(const EffPlan* plan, const float* y, const void* fhat, const void* xhat, float* u,
                       float* fz, float alpha, float beta, int batch, void* stream);

/* eff_adjoint of mask .* y (mask [batch, sy0, sy1]) without forming the
 * product: Ft(m y) of the multiplicative image step, vmbd_chimney.py:143. */
EFF_API int eff_adjoint_masked(const EffPlan* plan, const float* y, const float* mask, const void* fhat,
                       const void* xhat, float* gx, float* gf, int adj_mode, int batch, void* stream);

/* Chained calls without clears.  A call whose output is accumulated first
 * clears it with a small kernel that the call's own kernel overlaps (about
 * 1 us in a graph); loops that run many forward / adjoint pairs in one graph
 * (the MFBD frame) can instead have each accumulated output zeroed as a side
 * job of an earlier kernel that does not touch it, and its own call skip
 * the clear.
 * eff_forward_ex: eff_forward_image (operand EFF_OPERAND_IMAGE, spec =
 *   fhat) or eff_forward_psf (EFF_OPERAND_PSF, spec = xhat); sub
 *   (nullable, not aliasing y): y = EFF - sub, the residual against an
 *   observation sub, formed by the same kernel as in eff_forward_residual;
 *   flags
 *   EFF_OUT_ZEROED: y is already zero; zero_f[0, zero_nf) (float) and
 *   zero_d[0, zero_nd) (double), nullable, are cleared by the kernel for a
 *   later call and must not overlap anything this call reads or writes.
 * eff_adjoint_ex: eff_adjoint / eff_adjoint_residual (y_obs) /
 *   eff_adjoint_masked (mask) in one; flags EFF_OUT_ZEROED: gx and loss are
 *   already zero; EFF_LOSS_OF_Y (no y_obs, no mask): y is the residual, as
 *   eff_forward_residual leaves it, and loss (nullable) += 0.5 * sum y^2;
 *   EFF_AFTER_FORWARD: programmatic dependent launch after the preceding
 *   forward call (eff_loss_grad does this internally). */
EFF_API int eff_forward_ex(const EffPlan* plan, int operand, const float* u, const void* spec, float* y, const float* sub,
                   void* spec_out, int flags, float* zero_f, long long zero_nf, double* zero_d, int zero_nd,
                   int batch, void* stream);
EFF_API int eff_adjoint_ex(const EffPlan* plan, const float* y, const float* y_obs, const float* mask, const void* fhat,
                   const void* xhat, float* gx, float* gf, double* loss, int adj_mode, int flags, int batch,
                   void* stream);
/* eff_forward_both (sub NULL) / eff_forward_residual (sub = y_obs, not
 * aliasing y) with the same flags and side jobs as eff_forward_ex.
 * eff_loss_grad is: a clear of its residual buffer, this call with
 * EFF_OUT_ZEROED clearing gx and loss, eff_adjoint_ex with
 * EFF_OUT_ZEROED | EFF_LOSS_OF_Y. */
EFF_API int eff_forward_both_ex(const EffPlan* plan, const float* x, const float* f, const float* sub, float* y,
                        void* xhat_out, void* fhat_out, int flags, float* zero_f, long long zero_nf, double* zero_d,
                        int zero_nd, int batch, void* stream);

/* Online MFBD helpers (vmbd_chimney.py:110-182 with projected-gradient PSF
 * steps, optGPU.py:134-358):
 * eff_dots3: out[0] = sum u^2 (na terms), out[2] = sum v^2 (nb terms),
 *   out[1] = sum u v (min(na, nb) terms), u = a - ap, v = b - bp (ap/bp
 *   nullable), accumulated in double.
 * eff_pg_step: per PSF (K of n samples), f_prev <- f, g_prev <- g,
 *   f <- P_simplex(f - s g), with s from dots: mode 0 exact line search
 *   (<g,g> / ||Xg||^2 in dots[0], dots[2]), mode 1/2 Barzilai-Borwein
 *   <dx,dx>/<dx,dg> and <dx,dg>/<dg,dg> (optGPU.py:222-226); state[0] keeps
 *   the step and is reused when the curvature is not positive.
 * eff_max_nonneg: *out_bits = max(0, max a) as float bits (device word).
 * eff_mu_update: x *= max(num' / (den + tol), tol) with num' = num where
 *   num > floor_rel * max(num) (num_max_bits from eff_max_nonneg) and 0
 *   elsewhere, then x = min(x, max of x over the interior [border0,
 *   rows-border0) x [border1, cols-border1)) (vmbd_chimney.py:143-147).
 *   Where no data reaches a pixel num and den are 0 in exact arithmetic (the
 *   factor is tol) but FP32 transform noise well above tol = 1e-10; the
 *   floor (1e-6 in vmbd_gb300.mfbd) restores the exact-arithmetic factor.
 *   xmax_bits is a device scratch word.
 * flags EFF_OUT_ZEROED: out (eff_dots3) / xmax_bits (eff_mu_update) is
 * already zero; zero_f[0, zero_n) (nullable) is cleared as a side job, as in
 * eff_forward_ex. */
EFF_API int eff_dots3(const float* a, const float* ap, long long na, const float* b, const float* bp, long long nb,
              double* out, int flags, void* stream);
EFF_API int eff_pg_step(float* f, const float* g, float* f_prev, float* g_prev, int K, int n, const double* dots,
                int mode, float* state, float* zero_f, long long zero_n, void* stream);
EFF_API int eff_max_nonneg(const float* a, long long n, unsigned* out_bits, void* stream);
EFF_API int eff_mu_update(float* x, const float* num, const float* den, float tol, int rows, int cols, int border0,
                  int border1, const unsigned* num_max_bits, float floor_rel, unsigned* xmax_bits, int flags,
                  float* zero_f, long long zero_n, void* stream);

/* Uneven batches in one persistent launch (e.g. 24 x 256^2 + 24 x 384x512 +
 * 16 x 1024^2 images):
 * images of up to 8 geometries (one plan each, counts[c] images of plan c,
 * stored back to back per class) are processed by one kernel launch per
 * direction.  The batch keeps a device work list of (class, image, patch)
 * items, largest FFT frame first, walked statically by a grid of 2-CTA
 * clusters (one CTA per SM).  Per-class arguments are arrays of n_classes
 * device pointers (host arrays); outputs accumulated with atomics (y, gx,
 * loss) are cleared by the call. */
typedef struct EffBatch EffBatch;
EFF_API int eff_batch_create(const EffPlan* const* plans, const int* counts, int n_classes, EffBatch** batch);
EFF_API int eff_batch_destroy(EffBatch* batch);
EFF_API int eff_batch_items(const EffBatch* batch);
/* eff_forward_both over the batch: x, f -> y (+ both spectra, nullable). */
EFF_API int eff_batch_forward_both(const EffBatch* batch, const float* const* x, const float* const* f, float* const* y,
                           void* const* xhat_out, void* const* fhat_out, void* stream);
/* eff_forward_residual over the batch: r = EFF(x, f) - y_obs per image. */
EFF_API int eff_batch_forward_residual(const EffBatch* batch, const float* const* x, const float* const* f,
                               const float* const* y_obs, float* const* r, void* const* xhat_out,
                               void* const* fhat_out, void* stream);
/* eff_adjoint_residual over the batch; y_obs nullable: y is already the
 * residual (eff_batch_forward_residual) and loss (nullable) = 0.5 * sum y^2;
 * gx needs fhat, gf needs xhat. */
EFF_API int eff_batch_adjoint_residual(const EffBatch* batch, const float* const* y, const float* const* y_obs,
                               const void* const* fhat, const void* const* xhat, float* const* gx,
                               float* const* gf, double* const* loss, void* stream);

/* How many CTAs process one patch, for all plans of the process:
 * 0 (default) per call -- a 2-CTA thread-block cluster when one CTA's frame
 * does not fit in shared memory or when twice the grid still fits on the
 * GPU's SMs at once; 1 always one CTA (where it fits); 2 always a cluster. */
EFF_API int eff_set_cluster_mode(int mode);

/* Error bits the plan's kernels recorded on the device (EFF_DEVERR_*), read
 * after waiting for all work on the current device; clear != 0 resets them.
 * EFF_DEVERR_COPY_TIMEOUT: a bulk copy into shared memory did not complete
 * within the kernel's wait limit (that call's results are not valid). */
#define EFF_DEVERR_COPY_TIMEOUT 1
EFF_API int eff_plan_device_errors(const EffPlan* plan, int* flags, int clear);

/* Kernels that multiply by cached spectra (adjoints, forwards from a cached
 * spectrum, deconvolution) either copy their columns of the spectra into
 * shared memory with the bulk-copy engine at kernel start, where the CTA's
 * shared memory allows, or read them from global memory.  2 (default): the
 * deconvolution copies (its spectra usually come from HBM), the rest read (a
 * loss/gradient step's adjoint finds its spectra in L2); 1: every such
 * kernel copies; 0: none does.  For all plans of the process. */
EFF_API int eff_set_spectrum_staging(int on);

/* 1 (default): kernels that read the image (image spectrum, forwards from x)
 * copy each CTA's rows of the patch window into shared memory with one
 * tensor-engine (TMA) copy at kernel start, where x is 16-byte aligned and
 * the image width and the patch hop are multiples of 4; 0: every lane loads
 * its own values.  For all plans of the process. */
EFF_API int eff_set_image_tile(int on);

/* Testing hook: overwrite the device a plan records as its own, so that a
 * test can check that calls on a mismatched device are refused before any
 * work is queued.  Not for production use. */
EFF_API int eff_test_plan_set_device(EffPlan* plan, int device);

/* Message for the last non-OK status returned on this thread. */
EFF_API const char* eff_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* VMBD_EFF_H */
