/*
 * temgym_gb300.h - C ABI of the GB300 (sm_103a) implementation of TemGymCore's
 * batched paraxial ray propagation and Gaussian-beamlet detector field.
 *
 * The reference (temgym_core, pure Python on JAX) has no FFI: its "plugin
 * API" is Python duck typing.  Each entry point below replaces a Python call
 * site of the reference (cited per function); the Python package
 * temgymcore_gb300 binds them with ctypes.
 *
 * Conventions
 *   - Every function returns an int status: TG_OK (0) or a negative TG_ERR_*.
 *   - Buffers marked "device" are caller-owned CUDA device pointers; the
 *     library allocates nothing except where a function says otherwise.
 *   - `stream` is a cudaStream_t passed as void*; NULL is the legacy stream.
 *     Calls enqueue work and return without synchronising, so they can be
 *     captured into a CUDA graph.
 *   - Kernels never trap: a device-side problem (non-finite coordinate in a
 *     histogram, bad table entry, exhausted wait) sets bits in a device error
 *     word, read back with tg_get_error_word().
 *   - Ray state is float32 structure-of-arrays; pathlength, phases and ABCD
 *     matrices are float64.
 */
#ifndef TEMGYM_GB300_H
#define TEMGYM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define TG_OK 0
#define TG_ERR_INVALID (-1)     /* null pointer, bad size, bad enum        */
#define TG_ERR_UNSUPPORTED (-2) /* component kind / option not supported  */
#define TG_ERR_ALIGN (-3)       /* pointer alignment requirement violated  */
#define TG_ERR_CUDA (-4)        /* a CUDA runtime call failed              */
#define TG_ERR_TOO_LARGE (-5)   /* size beyond a stated maximum            */
#define TG_ERR_WORKSPACE (-6)   /* caller workspace too small              */

/* device error-word bits (tg_get_error_word) */
#define TG_EW_NONFINITE 0x1u    /* non-finite coordinate met by a binner   */
#define TG_EW_TABLE 0x2u        /* out-of-range entry in a packed table    */
#define TG_EW_TIMEOUT 0x4u      /* a bounded wait gave up                  */
#define TG_EW_MMA 0x8u          /* tensor-core pipeline wait gave up       */

/* ---- component kinds (components.py) ---------------------------------- */
enum tg_kind {
  TG_PLANE = 0,     /* Plane, Detector, ScanGrid, Source: identity        */
  TG_LENS = 1,      /* p[0] = focal_length                                 */
  TG_SCANNER = 2,   /* p[0..3] = scan_pos_x, scan_pos_y, tilt_x, tilt_y     */
  TG_DESCANNER = 3, /* p[0..3] = scan pos/tilt; p[4..19] = 4x4 matrix M     */
                    /* (rows x,y,dx,dy; cols spx,spy,stx,sty, row-major);  */
                    /* p[20..23] = offsets.  Delta = M s + off - s.  The    */
                    /* reference's 12 coefficients are M[:,0:2] and off    */
                    /* with M[:,2:4] = 0.                                  */
  TG_DEFLECTOR = 4, /* p[0..1] = def_x, def_y                              */
  TG_BIPRISM = 5,   /* p[0] = def_x                                        */
  TG_ROTATOR = 6,   /* p[0] = angle in degrees                             */
  TG_THICKLENS = 7, /* z = z_po; p[0] = focal_length; p[1] = z_pi          */
  TG_APERTURE = 8,  /* p[0] = radius; p[1..2] = centre x, y (extension)    */
  TG_ABERLENS = 9   /* AberratedLensKrivanek: p[0] = focal_length;        */
                    /* p[1..25] = C10, C12, phi12, C21, phi21, C23, phi23, */
                    /* C30, C32, phi32, C34, phi34, C41, phi41, C43, phi43,*/
                    /* C45, phi45, C50, C52, phi52, C54, phi54, C56, phi56 */
                    /* (aberrations.py:5-31 order).  Forward trace, scan,  */
                    /* ABCD and field prep only (adjoint, batched: status  */
                    /* TG_ERR_UNSUPPORTED); at most 4 per model.           */
};

/* component flag: scan position comes from the probe (tg_scan_*) */
#define TG_FLAG_PER_PROBE 0x1

typedef struct tg_component {
  int32_t kind;  /* enum tg_kind */
  int32_t flags; /* TG_FLAG_* */
  double z;      /* axial position in metres (ThickLens: z_po) */
  double p[32];  /* kind-specific parameters, see enum tg_kind */
} tg_component;

/* free-space propagator between components (propagator.py:43-116) */
#define TG_PROP_PARAXIAL 0 /* FreeSpaceParaxial: x += dx d, pathlength += d          */
#define TG_PROP_DIRCOS 1   /* FreeSpaceDirCosine: N = sqrt(1 + dx^2 + dy^2),         */
                           /* x += dx d / N^2, pathlength += d N.  Forward trace,    */
                           /* adjoint, scan and ABCD; batched / field: unsupported   */

typedef struct tg_model {
  int32_t n_components;            /* <= TG_MAX_COMPONENTS */
  int32_t propagator;              /* TG_PROP_* (0 = paraxial) */
  const tg_component *components;  /* host pointer */
} tg_model;

#define TG_MAX_COMPONENTS 60

/* Structure-of-arrays rays (ray.py:8-45).  x, y, dx, dy: device float32 of
 * length n.  z and pathlength: device float64 arrays, or NULL to use the
 * uniform *_scalar value.  amplitude: optional device float32 (NULL = none).
 */
typedef struct tg_rays {
  int64_t n;
  float *x, *y, *dx, *dy;
  double *z;
  double z_scalar;
  double *pathlength;
  double pl_scalar;
  float *amplitude;
} tg_rays;

/* Detector pixel map (grid.py:51-63,120-153).  m is the first two rows of
 * the float64 metres->pixels matrix; py = (m[0]*y + m[1]*x) + m[2],
 * px = (m[3]*y + m[4]*x) + m[5], rounded half-to-even to int32. */
typedef struct tg_grid {
  int32_t h, w;
  double m[6];
} tg_grid;

/* ---- library --------------------------------------------------------- */
/* Version string of this library. */
const char *tg_version(void);
/* Human-readable text for a status code. */
const char *tg_status_string(int status);
/* Read (and optionally clear) the device error word of the current device;
 * synchronises the device. */
int tg_get_error_word(uint32_t *out, int clear);

/* Read and clear the device error word (0xffffffff if it could not be read). */
uint32_t tg_get_last_error_word(void);

/*
 * tg_selftest_add_f64_f32 - diagnostics: the pathlength rounding the trace
 * kernels use (base + float32 part, rounded to nearest even with float32 and
 * integer operations) next to the float64 add, over n device pairs:
 * fast[i] = emulated b[i] + p[i], ref[i] = float64 b[i] + (double)p[i].  The
 * two must agree bit for bit.  No reference counterpart.
 */
int tg_selftest_add_f64_f32(const double *b, const float *p, double *fast, double *ref,
                            int64_t n, void *stream);

/* ---- ray chain -------------------------------------------------------- */
/*
 * tg_trace_fwd - fused forward trace (+ optional pixel binning + histogram).
 * Replaces run.py:85-116 run_to_end (with run_iter's always-inserted
 * propagator, run.py:75-82), followed optionally by grid.py:120-153
 * Detector.metres_to_pixels and grid.py:231-280 Detector.into_image.
 *   out:   output rays (x, y, dx, dy float32; pathlength float64 if non-NULL;
 *          amplitude if both in/out amplitude non-NULL).  Output z is
 *          uniform and is returned in *z_out (may be NULL).
 *   grid:  NULL = no binning.  pix_y/pix_x (device int32, length n) may be
 *          NULL.  hist (device, grid h*w) may be NULL; hist_i64 selects
 *          int64 (reference dtype) or int32 counters.  hist is ADDED to.
 */
int tg_trace_fwd(const tg_model *model, const tg_rays *in, tg_rays *out,
                 double *z_out, const tg_grid *grid, int32_t *pix_y,
                 int32_t *pix_x, void *hist, int32_t hist_i64, void *stream);

/*
 * tg_trace_image - tg_trace_fwd with a caller workspace for the histogram.
 * Same replacement (run.py:85-116 + grid.py:120-153 + grid.py:231-280,
 * Detector.into_image) and same results: the histogram is ADDED to.  When
 * tg_trace_image_workspace(n, grid) is non-zero and workspace holds that many
 * bytes (16-byte aligned device memory), each SM keeps a private copy of the
 * detector in shared memory and the copies are summed at the end (one shared
 * atomic per hit instead of one global atomic); otherwise the call
 * is tg_trace_fwd.  The workspace query is 0 for detectors above ~100k pixels
 * or fewer than 32 rays per pixel, where global atomics are the better choice.
 */
size_t tg_trace_image_workspace(int64_t n, const tg_grid *grid);
int tg_trace_image(const tg_model *model, const tg_rays *in, tg_rays *out,
                   double *z_out, const tg_grid *grid, int32_t *pix_y,
                   int32_t *pix_x, void *hist, int32_t hist_i64, void *workspace,
                   size_t ws_bytes, void *stream);

/*
 * tg_bin - metres->pixels + histogram for existing rays (no trace).
 * Replaces grid.py:120-153 and grid.py:231-280 (+ utils.py:83-114).
 * mask: optional device uint8 (0 = do not count), may be NULL.
 */
int tg_bin(int64_t n, const float *x, const float *y, const uint8_t *mask,
           const tg_grid *grid, int32_t *pix_y, int32_t *pix_x, void *hist,
           int32_t hist_i64, void *stream);

/*
 * tg_hist_workspace - workspace bytes for the per-SM shared-memory histogram
 * path of tg_trace_image, tg_bin_image and tg_hist_pixels: non-zero for
 * detectors of at most 102,400 pixels with at least 32 rays per pixel, 0
 * otherwise (the calls then use global atomics).  tg_trace_image_workspace
 * is this query for a grid.
 */
size_t tg_hist_workspace(int64_t n, int32_t h, int32_t w);

/* tg_bin_image - tg_bin with the histogram workspace (same results). */
int tg_bin_image(int64_t n, const float *x, const float *y, const uint8_t *mask,
                 const tg_grid *grid, int32_t *pix_y, int32_t *pix_x, void *hist,
                 int32_t hist_i64, void *workspace, size_t ws_bytes, void *stream);

/*
 * tg_hist_pixels - histogram of existing integer pixel indices.
 * Replaces grid.py:231-280 Detector.into_image given (pixels_y, pixels_x)
 * (utils.py:83-114): indices outside [0, h) x [0, w) are dropped, the counts
 * are ADDED to hist [h][w].  idx_i64: indices are int64 (else int32);
 * hist_i64: counts are int64 (else int32).  workspace as tg_hist_workspace.
 */
int tg_hist_pixels(int64_t n, const void *pix_y, const void *pix_x, int32_t idx_i64,
                   int32_t h, int32_t w, void *hist, int32_t hist_i64, void *workspace,
                   size_t ws_bytes, void *stream);

/*
 * tg_abcd_compose - float64 5x5 ABCD about a central ray, composed from the
 * per-step component matrices (host code, no GPU needed).
 * Replaces jax.jacobian(run_to_end) + utils.py:7-43 custom_jacobian_matrix
 * (README.md:224-234) and, with steps != NULL, run.py:150-179 solve_model
 * (steps receives 2*n_components row-major 5x5 matrices).
 * central: x, y, dx, dy, z of the central ray (biprism sign depends on it).
 */
int tg_abcd_compose(const tg_model *model, const double central[5],
                    double out[25], double *steps);

/*
 * tg_aber_monomials - the Krivanek wave aberration as a polynomial (host
 * code, no GPU needed): kc holds the 25 KrivanekCoeffs values in field order
 * (aberrations.py:5-31); w[28] receives the coefficient of ax^p ay^q of
 * W (aberrations.py:51-61) at index p * 7 - p * (p - 1) / 2 + q (p + q <= 6),
 * gx[21] / gy[21] (either may be NULL) those of dW/dax and dW/day
 * (aberrations.py:64-108) at p * 6 - p * (p - 1) / 2 + q (p + q <= 5).
 * The kernels evaluate the aberrated lens from these coefficients.
 */
int tg_aber_monomials(const double kc[25], double w[28], double *gx, double *gy);

/*
 * tg_trace_vjp - adjoint of tg_trace_fwd (reverse mode, forward state
 * recomputed per ray, nothing stored between the passes).
 * Replaces jax.grad / jax.vjp of run_to_end (README.md:113-160,
 * run.py:182-267 run_with_grads).
 *   gout:  upstream gradients (x, y, dx, dy float32; pathlength float64 or
 *          NULL = zero).  gin: gradients w.r.t. the input rays (any of its
 *          pointers may be NULL; gin->pathlength receives float64).
 *   raw:   device float64 [n_steps][4], n_steps = 2*n_components, ADDED to:
 *          per step the ray-summed adjoint quantities from which parameter
 *          gradients follow: propagator dL/dd; lens dL/df; scanner and
 *          descanner dL/d(offset x, y, dx, dy); deflector dL/d(def_x, def_y);
 *          biprism dL/d(def_x); rotator dL/d(angle in radians).
 *   workspace: device scratch of tg_trace_vjp_workspace(n) bytes.
 */
size_t tg_trace_vjp_workspace(int64_t n, const tg_model *model);

/*
 * tg_trace_adj - gradient of loss = sum_i |(x, y)_out,i - target_i|^2 for
 * one model in one call (forward, residual, adjoint): the reference's
 * jax.grad of a squared detector-position loss over run_to_end
 * (README.md:113-160).  target_x/y: device float32 [n].  dparams: device
 * float64 [2*n_components][4], OVERWRITTEN with the per-step sums of
 * tg_trace_vjp.  dray (may be NULL): gradients w.r.t. the input rays.
 * workspace: device, tg_trace_adj_workspace(n, model) bytes, 256-byte aligned.
 */
size_t tg_trace_adj_workspace(int64_t n, const tg_model *model);
int tg_trace_adj(const tg_model *model, const tg_rays *in, const float *target_x,
                 const float *target_y, double *dparams, tg_rays *dray, void *workspace,
                 size_t ws_bytes, void *stream);
int tg_trace_vjp(const tg_model *model, const tg_rays *in, const tg_rays *gout,
                 tg_rays *gin, double *raw, void *workspace, size_t ws_bytes,
                 void *stream);

/* ---- 4D-STEM scan batch ---------------------------------------------- */
/* Probe p sits at scan-grid pixel (row, col) = (p / cols, p % cols); its
 * scan position is y = (t[0]*row + t[1]*col) + t[2], x = (t[3]*row +
 * t[4]*col) + t[5] (the ScanGrid pixels->metres map, grid.py:155-182), or
 * positions[2p], positions[2p+1] (x, y; device float64) when non-NULL.
 * Every Scanner / Descanner flagged TG_FLAG_PER_PROBE takes that position. */
typedef struct tg_scan {
  int32_t n_probes;
  int32_t cols;
  double t[6];
  const double *positions;
} tg_scan;

/*
 * tg_scan_hist - per-probe detector images of one ray bundle.
 * Replaces the per-scan-position loop of run.py:85-116 run_to_end followed
 * by grid.py:231-280 Detector.into_image (one Python call per position in
 * the reference).
 *   bundle: rays leaving the source (uniform z), shared by every probe.
 *   hist:   device int32 [n_probes][h][w], OVERWRITTEN (dense images).
 *   probe_xy: optional device float32 [n_probes][2][n]: detector x then y.
 */
int tg_scan_hist(const tg_model *model, const tg_rays *bundle, const tg_scan *scan,
                 const tg_grid *grid, int32_t *hist, float *probe_xy, void *stream);

/* ---- transfer-matrix stacks (transfer.py:6-183) ----------------------- */
/*
 * tg_transfer_cumulative - host: the cumulative products of m row-major 5x5
 * matrices exactly as transfer.py:150-183 accumulate_matrices_cumulative
 * builds them: cumulative[0] = M[m-1], cumulative[k] = M[m-1-k] @
 * cumulative[k-1] (so cumulative[k] = M[m-1-k] @ ... @ M[m-1]).
 */
int tg_transfer_cumulative(int32_t m, const double *matrices, double *cumulative);

/*
 * tg_transfer_rays - transfer.py:6-53: every ray (device float64 [n][5],
 * rows x, y, dx, dy, 1) through each cumulative product of the m host
 * matrices (m <= 120): out (device float64 [n][m][5]).  m == 0 is invalid
 * (the reference raises IndexError).
 */
int tg_transfer_rays(int64_t n, const double *rays, int32_t m, const double *matrices,
                     double *out, void *stream);

/*
 * tg_transfer_rays_pt_src - transfer.py:56-112: rays from the point (x0, y0)
 * with slopes (slopes_x[k], slopes_y[k]) (device float64) through one host
 * 5x5 matrix: out (device float64 [4][n], rows x, y, dx, dy).
 */
int tg_transfer_rays_pt_src(double x0, double y0, int64_t n, const double *slopes_x,
                            const double *slopes_y, const double *matrix, double *out,
                            void *stream);

/* ---- ray sources and beam decomposition ------------------------------- */
/*
 * tg_source_count - host: number of rays tg_source_generate writes for
 * num_approx: the concentric-ring total of utils.py:117-175 (random = 0) or
 * exactly num_approx (random = 1).
 */
int tg_source_count(int64_t num_approx, int32_t random, int64_t *n_rays);

/*
 * tg_source_generate - Source.generate_array (source.py:36-188) on the GPU:
 * out (device float64 [n][5], rows x, y, dx, dy, 1; capacity >= the count
 * above).  kind 0 = PointSource (extent = semi_conv: slopes on the disc,
 * positions at the offset), 1 = ParallelBeam (extent = radius: positions on
 * the disc plus the offset, zero slopes).  random = 0: the reference's
 * concentric rings, ray for ray (its running-angle recurrence included);
 * random = 1: uniform in the disc from a hash of (seed, index) - the
 * reference's distribution, not its NumPy draws.
 */
int tg_source_generate(int32_t kind, int32_t random, int64_t num_approx, uint64_t seed,
                       double extent, double off_x, double off_y, double *out, int64_t capacity,
                       void *stream);

/*
 * tg_decompose_q_inv - gaussian.py:35-89 for n beams: q_inv (device complex128
 * [n][2][2], re/im interleaved), wavelength (device float64 [n] or NULL =
 * wavelength_scalar) -> waist, radii (device float64 [n][2]: major axis first)
 * and theta (device float64 [n]).  theta is the reference's up to a multiple
 * of pi (an eigenvector's sign is a solver convention; Q^-1 is unchanged).
 */
int tg_decompose_q_inv(int64_t n, const double *q_inv, const double *wavelength,
                       double wavelength_scalar, double eps, double *waist, double *radii,
                       double *theta, void *stream);

/*
 * tg_inplace_sum - inplace_sum (utils.py:83-114): buffer[py, px] += frame[i]
 * for every hit i with mask[i] != 0 (mask NULL: all) and (py, px) inside the
 * h x w buffer (row-major, device).  pix_y / pix_x: device int32, or int64
 * when idx_i64.  dtype of frame and buffer: 0 int32, 1 int64, 2 float32,
 * 3 float64; frame NULL adds 1.  Integer buffers are exact; float buffers
 * round per add in the order the atomics land.
 */
int tg_inplace_sum(int64_t n, const void *pix_y, const void *pix_x, int32_t idx_i64, const uint8_t *mask,
                   const void *frame, int32_t dtype, int32_t h, int32_t w, void *buffer, void *stream);

/*
 * The beamlet field from per-beam ABCD blocks at arbitrary sample points
 * (complex128 out, float64 throughout, deterministic):
 *
 * tg_propagate_misaligned_gaussian - propagate_misaligned_gaussian_jax_scan
 *   (gaussian.py:319-337, _beam_field gaussian.py:276-316).  Device inputs:
 *   amp (complex128 [n]), phase_offset ([n], radians), q1_inv (complex128
 *   [n][2][2]), a, b, c, d (float64 [n][2][2]), e, f, r1m, theta1m ([n][2]),
 *   k ([n]); r2 ([n_points][2]: x, y) -> out (complex128 [n_points]).
 * tg_evaluate_misaligned_input_gaussian -
 *   evaluate_misaligned_input_gaussian_jax_scan (gaussian.py:410-427,
 *   _input_beam_field gaussian.py:402-409): the same without a, b, c, d, e, f.
 * Workspace: tg_misaligned_gaussian_workspace(n, n_points) bytes, 16-byte
 * aligned.  B^-1 and Q1 are zeroed where singular, as the reference does.
 */
size_t tg_misaligned_gaussian_workspace(int64_t n_beams, int64_t n_points);
int tg_propagate_misaligned_gaussian(int64_t n, const double *amp, const double *phase_offset,
                                     const double *q1_inv, const double *a, const double *b,
                                     const double *c, const double *d, const double *e, const double *f,
                                     const double *r1m, const double *theta1m, const double *k,
                                     int64_t n_points, const double *r2, double *out, void *workspace,
                                     size_t ws_bytes, void *stream);
int tg_evaluate_misaligned_input_gaussian(int64_t n, const double *amp, const double *phase_offset,
                                          const double *q1_inv, const double *r1m, const double *theta1m,
                                          const double *k, int64_t n_points, const double *r1, double *out,
                                          void *workspace, size_t ws_bytes, void *stream);

/*
 * tg_beam_q_inv - GaussianRay.q_inv and .Q_inv (gaussian.py:138-177) for n
 * beams: waist, radii (device float64 [n][2]; an infinite radius is a flat
 * wavefront), wavelength / theta (device float64 [n] or NULL = the scalar)
 * -> q_xy (device complex128 [n][2]: 1/qx, 1/qy; or NULL) and q_inv (device
 * complex128 [n][2][2] = R(theta) diag(1/qx, 1/qy) R(theta)^T; or NULL).
 */
int tg_beam_q_inv(int64_t n, const double *waist, const double *radii, const double *wavelength,
                  double wavelength_scalar, const double *theta, double theta_scalar,
                  double *q_xy, double *q_inv, void *stream);

/*
 * tg_qinv_abcd - Qinv_ABCD (gaussian.py:92-96) for n systems:
 * out = (A + B Q)^-1 (C + D Q), q_inv and out device complex128 [n][2][2],
 * A, B, C, D device float64 [n][2][2].  Solved by 2x2 LU with partial
 * pivoting, as linalg.solve does; a singular A + B Q gives inf / nan.
 */
int tg_qinv_abcd(int64_t n, const double *q_inv, const double *a, const double *b, const double *c,
                 const double *d, double *out, void *stream);

/*
 * tg_beam_profile - the Gaussian-beam helpers (gaussian.py:13-28, 99-109)
 * elementwise over n entries (device float64 [n] inputs, NULL where unused):
 *   z_r   = zR(w0, wavelength), or the given z_r_in copied;
 *   w_z   = w_z(w0, z, zR) and r = R(z, zR), with zR = z_r_in when given,
 *           else zR(w0, wavelength);
 *   q_inv = q_inv(z, w0, wavelength) (complex128 [n]; z_r_in must be NULL).
 * Each output may be NULL; an output whose inputs are missing is
 * TG_ERR_INVALID.  |z| < 1e-10 is the focus (R = inf).
 */
int tg_beam_profile(int64_t n, const double *z, const double *w0, const double *wavelength,
                    const double *z_r_in, double *z_r, double *w_z, double *r, double *q_inv,
                    void *stream);

/*
 * tg_gaussian_beam - gaussian_beam (gaussian.py:31-32) elementwise:
 * out = exp(1j k ((x + offset_x)^2 + (y + offset_y)^2) / 2 q_inv); x, y, k,
 * offsets device float64 [n], q_inv and out device complex128 [n].
 */
int tg_gaussian_beam(int64_t n, const double *x, const double *y, const double *q_inv, const double *k,
                     const double *offset_x, const double *offset_y, double *out, void *stream);

/* ---- many models in one persistent launch ------------------------------ */
typedef struct tg_batch_info {
  size_t plan_bytes;       /* bytes of the packed plan (copy it to the device) */
  size_t workspace_bytes;  /* device workspace for tg_batch_run              */
  int32_t n_tiles;         /* >= 1 per model (an empty model has one empty tile) */
  int32_t total_steps;     /* sum over models of 2 * n_components           */
  int64_t total_rays;
  int32_t max_steps;       /* largest 2 * n_components of one model         */
  int32_t max_moments;     /* largest adjoint moment count of one model     */
  int32_t n_models;
  int64_t partial_doubles; /* workspace layout: per-tile moment partials    */
  int64_t moment_doubles;  /* per-model moments                             */
  int32_t max_record_floats; /* largest per-model forward record (shared memory) */
} tg_batch_info;

/* Rays of all models concatenated in model order (device float32).  The
 * output coordinates are each model's chain composed in float64 on the host
 * (one affine map plus one offset per biprism sign) and applied to the input
 * ray in float32; the per-ray pathlength terms, biprism signs and aperture
 * tests come from the step-by-step float32 chain.  out_alive (device uint8,
 * may be NULL) receives 1 for a ray that every aperture passes, else 0; a
 * blocked ray keeps its traced coordinates.  With target_x/target_y (device
 * float32, may be NULL = forward only) the adjoint of
 *   loss = sum over alive rays of |(x, y)_out - target|^2
 * runs too: raw (device float64 [total_steps][4], OVERWRITTEN) receives each
 * model's per-step sums (the quantities of tg_trace_vjp), model m's steps
 * starting at 2 * (components of models 0..m-1), and loss (device float64
 * [n_models], may be NULL; needs targets) each model's loss.  The adjoint is
 * evaluated from per-model moments of the rays (the loss reaches every step
 * through the chain's ray-independent linear part), so it costs a few
 * multiply-adds per ray. */
typedef struct tg_batch_io {
  const float *x, *y, *dx, *dy;
  float *out_x, *out_y, *out_dx, *out_dy;
  double *out_pathlength;
  const float *target_x, *target_y;
  double *raw;
  uint8_t *out_alive; /* may be NULL */
  double *loss;       /* may be NULL */
} tg_batch_io;

/*
 * tg_batch_plan - pack n_models models (host) with n_rays[m] rays each and
 * input z z_in[m] (NULL = 0) into one plan of tiles of tile_rays rays.  Host
 * only: with plan == NULL fills *info (sizes); otherwise writes the plan into
 * the host buffer plan (info->plan_bytes) for the caller to copy to the
 * device.  Replaces a Python loop of run_to_end (run.py:85-116) per model.
 * Each model is composed on the host in float64 into closed forms over its
 * input ray and biprism signs (output map, pathlength form, the rows of each
 * biprism / aperture decision).  Statuses: TG_ERR_UNSUPPORTED for an
 * aberrated lens, per-probe scan positions or direction-cosine propagation;
 * TG_ERR_TOO_LARGE for a model with more than 16 biprisms or a record of
 * more than 8192 floats (about 60 components of which 16 biprisms and the
 * rest apertures).
 */
int tg_batch_plan(int32_t n_models, const tg_model *models, const int64_t *n_rays,
                  const double *z_in, int32_t tile_rays, void *plan, size_t plan_bytes,
                  tg_batch_info *info);

/*
 * tg_batch_run - one persistent launch over every tile of the plan (device
 * copy), forward and (with targets) adjoint; the CTA that completes a model's
 * last tile reduces that model's tile partials in tile order (deterministic)
 * and writes its per-step sums, so nothing else is launched besides one
 * memset of the work counters.  block in {128, 256, 512}; rays_per_thread in
 * {1, 2, 4}.  workspace: device, info->workspace_bytes, 256-byte aligned.
 * Statuses: TG_ERR_INVALID for a loss pointer without targets.
 */
int tg_batch_run(const void *plan_dev, const tg_batch_info *info, const tg_batch_io *io,
                 int32_t block, int32_t rays_per_thread, void *workspace, size_t ws_bytes,
                 void *stream);

/*
 * tg_batched_trace - tg_batch_plan + tg_batch_run in one call: the plan is
 * built on the host, copied into the front of the caller's device workspace
 * (tg_batched_trace_workspace bytes, 256-byte aligned; the call synchronises
 * the stream after that copy, so it is not for graph capture) and run with
 * tiles of 4,096 rays, 256 threads x 2 rays.
 */
size_t tg_batched_trace_workspace(int32_t n_models, const tg_model *models, const int64_t *n_rays,
                                  const double *z_in);
int tg_batched_trace(int32_t n_models, const tg_model *models, const int64_t *n_rays,
                     const double *z_in, const tg_batch_io *io, void *workspace, size_t ws_bytes,
                     void *stream);

/* ---- 4D-STEM calibration fit (device-resident parameters) -------------- */
/* Model: bundle at z = 0 -> Scanner + Descanner at z = defocus with the
 * probe's scan position (ScanGrid of rows x cols, centre 0) -> Lens(f) at
 * z = defocus + lens_gap -> Detector at z = defocus + camera_length.
 * theta (device float64 [21]): f, defocus, camera_length, scan rotation
 * (degrees), scan step, then the 4x4 descan matrix M row-major (rows x, y,
 * dx, dy; columns scan x, scan y, tilt x, tilt y).  Probe p sits at scan
 * pixel (p / cols, p % cols). */
typedef struct tg_stem_fit {
  int32_t n_rays, rows, cols;
  const float *x, *y, *dx, *dy;      /* device bundle [n_rays] */
  const float *target_x, *target_y;  /* device [rows*cols][n_rays] */
  double lens_gap;
} tg_stem_fit;

/* Workspace bytes of tg_stem_fit_forward / tg_stem_fit_loss_grad. */
size_t tg_stem_fit_workspace(int32_t n_probes);

/* Detector positions of every (probe, ray) at theta (device float32
 * [rows*cols][n_rays] each).  Replaces the per-probe run_to_end loop. */
int tg_stem_fit_forward(const tg_stem_fit *cfg, const double *theta, float *det_x,
                        float *det_y, void *workspace, size_t ws_bytes, void *stream);

/*
 * tg_stem_fit_loss_grad - out (device float64 [22]): out[0] = sum over probes
 * and rays of the squared detector-position residual, out[1..21] = d out[0] /
 * d theta.  One fused forward + adjoint pass per ray, deterministic
 * reductions.  Replaces jax.value_and_grad of a loss over run_to_end
 * (README.md:113-160).
 */
int tg_stem_fit_loss_grad(const tg_stem_fit *cfg, const double *theta, double *out,
                          void *workspace, size_t ws_bytes, void *stream);

/* One Adam update of theta (device float64 [n], n <= 1024) from grad; m, v
 * (device float64 [n]) and the step counter t (device int64) persist across
 * calls so the update replays inside a CUDA graph.  scale (optional, device
 * float64 [n]) runs Adam in units of scale[i]; mask (optional, device uint8)
 * freezes entries with 0. */
int tg_adam_step(double *theta, const double *grad, double *m, double *v, int64_t *t, int32_t n,
                 double lr, double beta1, double beta2, double eps, const double *scale,
                 const uint8_t *mask, void *stream);

/*
 * tg_stem_fit_step - one whole optimisation step in two launches:
 * tg_stem_fit_loss_grad into out, then the tg_adam_step update of the 21
 * parameters (theta updated in place, gradients out[1..21]), applied by the
 * reduction block that completes the last output.  Same results as the two
 * calls.  Replaces one step of an optax/Adam loop over jax.value_and_grad.
 */
int tg_stem_fit_step(const tg_stem_fit *cfg, double *theta, double *out, double *m, double *v,
                     int64_t *t, double lr, double beta1, double beta2, double eps,
                     const double *scale, const uint8_t *mask, void *workspace, size_t ws_bytes,
                     void *stream);

/* ---- Gaussian-beamlet detector field ----------------------------------- */
/* Beamlets (GaussianRay, gaussian.py:113-177): central rays and beam shape,
 * all device arrays.  amplitude is complex64 (re, im pairs); waist_xy and
 * radii are [n][2] (x, y) with +inf radius = flat wavefront; wavelength and
 * theta (rad) may be NULL (uniform wavelength_scalar, theta 0). */
typedef struct tg_beams {
  int64_t n;
  const double *x, *y, *dx, *dy;
  double z;
  const double *pathlength;
  const float *amplitude;
  const double *waist_xy;
  const double *radii;
  const double *wavelength;
  double wavelength_scalar;
  const double *theta;
} tg_beams;

/* Detector pixel centres (grid.py:83-100): y = (t[0]*row + t[1]*col) + t[2],
 * x = (t[3]*row + t[4]*col) + t[5] (the pixels->metres transform). */
typedef struct tg_pixel_map {
  int32_t h, w;
  double t[6];
} tg_pixel_map;

#define TG_FIELD_DIRECT 0     /* any Q2 (astigmatic): fixed-point phase direct sum */
#define TG_FIELD_SEPARABLE 1  /* diagonal Q2, unrotated grid: split-BF16 tcgen05 GEMM */
#define TG_FIELD_DIRECT_F64 2 /* all-float64 direct sum (comparator)               */
#define TG_EW_NONSEPARABLE 0x10u /* separable method given a non-separable beam */

/* Workspace bytes for tg_field_prep + tg_field_eval(method) (256-aligned). */
size_t tg_field_workspace(int64_t n_beams, int32_t h, int32_t w, int32_t method);

/*
 * tg_field_prep - per-beam float64 preparation into the workspace: ABCD of
 * each central ray (gaussian.py:234-249), Q1^-1 and Q2^-1 (gaussian.py:92-96,
 * 138-177), prefactor and the per-pixel phase polynomial (gaussian.py:276-316),
 * exact reduction of k*pathlength mod 2*pi.  flags (device int32, may be
 * NULL): bit 0 set when some beam is not separable.
 */
int tg_field_prep(const tg_model *model, const tg_beams *beams, const tg_pixel_map *pm,
                  void *workspace, size_t ws_bytes, int32_t *flags, void *stream);

/*
 * tg_field_prep_input - the same records for the field of the beams in their
 * own plane, sampled on the pixel map (evaluate_gaussian_input_image,
 * gaussian.py:372-427): per pixel r1 and beam,
 *   amplitude * exp(i (k/2) ((r1 - r1m)^T Q1^-1 (r1 - r1m) + 2 (r1 - r1m).theta1m)) * exp(i k pl).
 * No model and no ABCD; tg_field_eval then sums the beams exactly as for the
 * detector field (the separable method applies when Q1^-1 has no xy term).
 */
int tg_field_prep_input(const tg_beams *beams, const tg_pixel_map *pm, void *workspace,
                        size_t ws_bytes, int32_t *flags, void *stream);

/*
 * tg_field_eval - the field sum over beams at every detector pixel into out
 * (device complex64 [h][w], overwritten).  Replaces gaussian.py:319-369
 * propagate_misaligned_gaussian_jax_scan + map_reduce (and the reshape in
 * gaussian.py:257-273 make_gaussian_image).  Uses the records written by
 * tg_field_prep into the same workspace.
 */
int tg_field_eval(int32_t method, int64_t n_beams, const tg_pixel_map *pm, float *out,
                  void *workspace, size_t ws_bytes, void *stream);

/* tg_field_prep + tg_field_eval(TG_FIELD_DIRECT / TG_FIELD_SEPARABLE) in one
 * call; workspace as for tg_field_eval with that method. */
int tg_field_direct(const tg_model *model, const tg_beams *beams, const tg_pixel_map *pm,
                    float *out, void *workspace, size_t ws_bytes, void *stream);
int tg_field_separable(const tg_model *model, const tg_beams *beams, const tg_pixel_map *pm,
                       float *out, void *workspace, size_t ws_bytes, void *stream);

/* ---- beamlet field adjoint --------------------------------------------- */
/* Gradients of a real loss L of the detector field F (complex64 [h][w]) with
 * respect to the beams and the model.  Every pointer may be NULL (not
 * computed); all device memory, OVERWRITTEN. */
typedef struct tg_field_grads {
  float *amplitude;   /* complex64 pairs [n]: dL/dRe a + i dL/dIm a          */
  double *pathlength; /* [n]                                                  */
  double *x, *y, *dx, *dy; /* [n]: the central rays                           */
  double *raw;        /* [2 * n_components][4]: per-step sums, the layout of
                         tg_trace_vjp (propagator distance; lens focal length;
                         deflector def_x, def_y; biprism def_x; scanner /
                         descanner shifts x, y, dx, dy; rotator angle in rad) */
} tg_field_grads;

/*
 * tg_field_vjp - adjoint of tg_field_prep + tg_field_eval (make_gaussian_image,
 * gaussian.py:225-316, under jax.grad / jax.vjp).  grad: device complex64
 * [h][w], dL/dRe F + i dL/dIm F (PyTorch's gradient of a complex tensor).
 * Per beam the field is amp * exp(log pref + i k pl + i Phi(row, col)) with
 * Phi a complex quadratic in the pixel indices; the call reduces conj(grad) *
 * field against the six monomials of Phi per beam (one pass over beams x
 * pixels) and applies the chain rule from Phi's coefficients to the beam and
 * model parameters in float64 (forward-mode dual numbers for the model's step
 * parameters, closed-form derivatives for the central ray, whose ABCD algebra
 * does not depend on it).  An aberrated lens in the model
 * returns TG_ERR_UNSUPPORTED.  workspace: device, tg_field_vjp_workspace(n,
 * h, w) bytes, 256-byte aligned.  Deterministic (fixed-order reductions).
 */
size_t tg_field_vjp_workspace(int64_t n_beams, int32_t h, int32_t w);
int tg_field_vjp(const tg_model *model, const tg_beams *beams, const tg_pixel_map *pm,
                 const float *grad, const tg_field_grads *out, void *workspace, size_t ws_bytes,
                 void *stream);

/*
 * tg_field_vjp_input - the same for the field of the beams in their own
 * plane (evaluate_gaussian_input_image, gaussian.py:372-409); out->raw must
 * be NULL (there is no model).
 */
int tg_field_vjp_input(const tg_beams *beams, const tg_pixel_map *pm, const float *grad,
                       const tg_field_grads *out, void *workspace, size_t ws_bytes, void *stream);

/*
 * tg_field_vjp_ex / tg_field_vjp_input_ex - tg_field_vjp / tg_field_vjp_input
 * with the per-beam moments formed by `method`: TG_FIELD_DIRECT (the pass
 * over beams x pixels above) or TG_FIELD_SEPARABLE (beams with diagonal Q2
 * on an unrotated grid, as the separable forward: the field factors into
 * row and column phasors, E_b(r, c) = V_b(r) U_b(c), so the moments come
 * from one split-BF16 complex GEMM on the tensor cores,
 * X_a[r][b] = sum_c conj(grad[r][c]) U_b(c) dc^a for a = 0, 1, 2, and a pass
 * over the rows with V_b(r) dr^k; a beam that is not separable sets
 * TG_EW_NONSEPARABLE).  Same outputs; workspace tg_field_vjp_workspace_ex
 * (the separable method holds the bf16 planes of conj(grad) and of the 3n
 * column factors and the h x 3n product).
 */
size_t tg_field_vjp_workspace_ex(int32_t method, int64_t n_beams, int32_t h, int32_t w);
int tg_field_vjp_ex(int32_t method, const tg_model *model, const tg_beams *beams, const tg_pixel_map *pm,
                    const float *grad, const tg_field_grads *out, void *workspace, size_t ws_bytes,
                    void *stream);
int tg_field_vjp_input_ex(int32_t method, const tg_beams *beams, const tg_pixel_map *pm, const float *grad,
                          const tg_field_grads *out, void *workspace, size_t ws_bytes, void *stream);

/*
 * tg_field_direct_noalloc - tg_field_prep + tg_field_eval(TG_FIELD_DIRECT)
 * in one call that allocates nothing.  No counterpart in the reference: it
 * exists for callers that cannot call cudaMalloc (an allocator owned by
 * another framework, a pre-sized memory pool, a host that forbids device
 * allocation after start-up).  Its scratch (beam records + partial images) is
 * a fixed 32 MiB array inside the library, held by every GPU that loads the
 * library until the process exits.  Limits: at most 32768 beams, and
 *   part(n) + 8 * h * w <= 33554432 bytes, with
 *   part(n) = R(R(R(96 n) + 128 n) + 256), R(v) = v rounded up to 256
 * (the float32 and float64 beam records, a status word, and one complex64
 * partial image; about 3.2 million pixels at 32768 beams and 4.2 million
 * with a handful of beams); larger requests return TG_ERR_TOO_LARGE before
 * any work.  When tg_field_direct's beam chunks would not all fit, the
 * beams are summed in fewer chunks, so results agree with it to float32
 * rounding, not bit for bit.  Per-beam preparation flags (tg_field_prep's flags) are not reported
 * here.  The array's device address is looked up (cudaGetSymbolAddress) on
 * every call made outside stream capture; a call while its stream is being
 * captured uses the address of the last uncaptured call on that device, so
 * make at least one call on each device before capturing one.  All calls
 * share the array: calls that overlap on the GPU (other streams, other
 * threads) race and must be serialised by the caller.
 * out: device complex64 [h][w], overwritten.
 */
int tg_field_direct_noalloc(const tg_model *model, const tg_beams *beams,
                            const tg_pixel_map *pm, float *out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* TEMGYM_GB300_H */
