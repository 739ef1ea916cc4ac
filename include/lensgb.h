/*
 * lensgb.h -- C ABI of the GB300 lens image-simulation library (liblensgb.so).
 *
 * The library replaces the XLA program that JAXtronomy builds for
 * ImageModel.image and the functions it calls:
 *   ImageModel.image                  jaxtronomy/ImSim/image_model.py:432-492
 *   ImageModel.likelihood_data_given_model  image_model.py:163-221
 *   LensModel.ray_shooting / alpha    jaxtronomy/LensModel/lens_model.py:237-252,353-381
 *                                     -> SinglePlane.ray_shooting/alpha single_plane.py:39-56,113-139
 *   LightModel.surface_brightness     jaxtronomy/LightModel/light_model_base.py:230-252
 *   Numerics.re_size_convolve         jaxtronomy/ImSim/Numerics/numerics.py:158-177
 *
 * Conventions
 *  - Every pointer named *_dev is a device pointer; the caller owns all
 *    buffers.  Arrays are dense, row-major and contiguous.
 *  - Every entry point is asynchronous on the given CUDA stream (a
 *    cudaStream_t passed as void*; NULL is the legacy default stream).
 *  - Every entry point returns a status code (LENSGB_OK == 0) and never aborts.
 *    lensgb_last_error() returns a thread-local description of the last
 *    failure on the calling thread.
 *  - A model handle owns device scratch and is used by one stream at a time.
 *
 * Per-system parameters are one row of doubles: the lens profiles' kwargs,
 * then the source profiles', then the lens-light profiles', each profile in
 * the order of its reference param_names (missing optional centres must be
 * filled with their default 0):
 *   SIE            theta_E e1 e2 center_x center_y                 (sie.py:40)
 *   NIE            theta_E e1 e2 s_scale center_x center_y         (nie.py:19)
 *   EPL            theta_E gamma e1 e2 center_x center_y           (epl.py:50)
 *   SHEAR          gamma1 gamma2 ra_0 dec_0                        (shear.py:16)
 *   CONVERGENCE    kappa ra_0 dec_0                                (convergence.py:15)
 *   NFW            Rs alpha_Rs center_x center_y                   (nfw.py:49)
 *   TNFW           Rs alpha_Rs r_trunc center_x center_y           (tnfw.py:27)
 *   NFW_ELLIPSE_CSE Rs alpha_Rs e1 e2 center_x center_y            (nfw_ellipse_cse.py:172)
 *   EPL_MULTIPOLE_M1M3M4 theta_E gamma e1 e2 center_x center_y a1_a delta_phi_m1
 *                  a3_a delta_phi_m3 a4_a delta_phi_m4            (epl_multipole_m1m3m4.py:415-428)
 *   SERSIC         amp R_sersic n_sersic center_x center_y         (sersic.py:27)
 *   SERSIC_ELLIPSE amp R_sersic n_sersic e1 e2 center_x center_y   (sersic_ellipse.py:25)
 */
#ifndef LENSGB_H
#define LENSGB_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define LENSGB_OK 0
#define LENSGB_ERR_INVALID 1     /* bad argument, shape or size            */
#define LENSGB_ERR_UNSUPPORTED 2 /* unknown profile code or option         */
#define LENSGB_ERR_OOM 3         /* device allocation failed               */
#define LENSGB_ERR_CUDA 4        /* kernel launch / runtime failure        */

/* ---- profile codes ------------------------------------------------------- */
#define LENSGB_LENS_SIE 1
#define LENSGB_LENS_NIE 2
#define LENSGB_LENS_EPL 3
#define LENSGB_LENS_SHEAR 4
#define LENSGB_LENS_NFW 5
#define LENSGB_LENS_TNFW 6
#define LENSGB_LENS_NFW_ELLIPSE_CSE 7
#define LENSGB_LENS_EPL_MULTIPOLE_M1M3M4 8
#define LENSGB_LENS_CONVERGENCE 9

#define LENSGB_LIGHT_SERSIC 1
#define LENSGB_LIGHT_SERSIC_ELLIPSE 2

/* ---- numerics ------------------------------------------------------------ */
#define LENSGB_PSF_NONE 0
#define LENSGB_PSF_PIXEL 1    /* zero-padded "same" convolution            */
#define LENSGB_PSF_GAUSSIAN 2 /* edge-padded "same" convolution            */

#define LENSGB_FP64 0       /* plain FP64 arithmetic throughout             */
#define LENSGB_FP32_SPLIT 1 /* FP32 bulk; FP64 set-up and FP64-accurate offsets */

#define LENSGB_MAX_PROFILES 8

/* flags of lensgb_image */
#define LENSGB_UNCONVOLVED 1   /* image(..., unconvolved=True)     */
#define LENSGB_NO_SOURCE 2     /* image(..., source_add=False)     */
#define LENSGB_NO_LENS_LIGHT 4 /* image(..., lens_light_add=False) */

typedef struct lensgb_model lensgb_model;

typedef struct {
    int n_lens;
    int lens_codes[LENSGB_MAX_PROFILES];
    int n_source;
    int source_codes[LENSGB_MAX_PROFILES];
    double deflection_scaling[LENSGB_MAX_PROFILES]; /* per source, 1 = none */
    int n_lens_light;
    int lens_light_codes[LENSGB_MAX_PROFILES];
    int nx, ny;            /* image columns, rows                               */
    int supersampling;     /* supersampling_factor (>= 1)                       */
    double transform_pix2angle[4]; /* row-major 2x2                             */
    double ra_at_xy_0, dec_at_xy_0;
    double flux_scaling;   /* ImageData.flux_scaling                             */
    double alpha_scaling;  /* SinglePlane alpha_scaling                          */
    int psf_type;          /* LENSGB_PSF_*                                       */
    int kernel_size;       /* odd side of the PSF kernel (0 for NONE)            */
    int precision;         /* LENSGB_FP64 or LENSGB_FP32_SPLIT                   */
    int supersampling_convolution; /* 1: convolve on the supersampled grid with a
                              kernel_size x kernel_size supersampled kernel, then
                              re-bin (SubgridKernelConvolution without a low-res
                              part / GaussianConvolution, convolution.py:100-166,
                              215-250); ignored when supersampling == 1     */
    int low_res_kernel_size; /* PIXEL with supersampling_convolution: side of the
                              pixel-scale part of a split kernel (0: none).  The PSF
                              of a system is then kernel_size^2 supersampled values
                              followed by low_res_kernel_size^2 pixel-scale values
                              (SubgridKernelConvolution, convolution.py:117-166) */
} lensgb_model_desc;

/* Build a model (the "compile" step of ImageModel.__init__,
 * image_model.py:27-150).  Validates codes and sizes; allocates nothing on the
 * device until the first call that needs it. */
int lensgb_model_create(const lensgb_model_desc* desc, lensgb_model** out);
int lensgb_model_destroy(lensgb_model* model);

/* Number of doubles per system row for this model. */
int lensgb_model_param_count(const lensgb_model* model);

/* NumericsSubFrame (numerics_subframe.py:20-200): compute only the n x n
 * sub-frame whose top-left pixel is (row0, col0) -- the bounding box of the
 * reference's flux_evaluate_indexes -- with the n x n evaluation mask `mask`
 * (host, row-major bytes, 0 = pixel not evaluated; NULL = all), convolve it as
 * an image of its own and return full images that are zero outside it.  As in
 * the reference, the sub-frame's pixel (0, 0) is placed at
 * map_pix2coord(row0, col0) (row index in the pixel-x slot, :185-190). */
int lensgb_model_set_subframe(lensgb_model* model, int row0, int col0, int n,
                              const unsigned char* mask);

/* Grow the model's device scratch to hold n_inst systems now, so that later
 * calls with at most n_inst systems allocate nothing (needed before capturing
 * those calls into a CUDA graph).  No counterpart in the reference. */
int lensgb_model_reserve(lensgb_model* model, int n_inst);

/* Launch shapes of a model's image calls.  ppt: pixels per thread of the ray
 * kernel (1, 2, 4 or 8); conv_tile_rows: output rows per tile of the FP32
 * convolution (a multiple of 4 in 32..64); 0 keeps the built-in choice.  They
 * change no result: every pixel's arithmetic is the same under any shape. */
int lensgb_model_set_tuning(lensgb_model* model, int ppt, int conv_tile_rows);

/* The autotuner: runs the model's image call on the caller's inputs (n_inst
 * systems, as lensgb_image) with every ray-kernel ppt in {1, 2, 4, 8} and every
 * convolution tile height in {32, 36, ..., 64} (FP32; FP64 has one shape),
 * timing each with CUDA events on `stream` (the minimum of three launches after
 * a warm-up), and keeps the fastest shapes in the model (the tuned ppt applies
 * to calls of at least a quarter of the tuned call's pixels; smaller calls keep
 * the built-in choice).  Synchronizes the stream; not for use while a graph is
 * being captured.  out_dev receives an image of the last run.  No counterpart
 * in the reference. */
typedef struct {
    int ppt;                  /* chosen ray-kernel pixels per thread             */
    int conv_tile_rows;       /* chosen convolution tile height (0: FP64 / none) */
    double ray_ms;            /* its prepare + ray + refine time                 */
    double conv_ms;           /* its convolution time                            */
    double ray_ms_builtin;    /* the same with the built-in shapes               */
    double conv_ms_builtin;
} lensgb_tune_result;

int lensgb_model_autotune(lensgb_model* model, const double* params_dev, int n_inst,
                          const void* psf_dev, long long psf_stride, void* out_dev, void* stream,
                          lensgb_tune_result* result);

/* FP32-split models only: pixels whose predicted FP32 error exceeds `tau`
 * (relative, per supersampled ray) are recomputed in FP64.  The prediction is
 * (sum_k I_k |d ln I_k / d beta|) * kappa * (|alpha_x| + |alpha_y|) / I_ray, with
 * kappa the FP32 relative error bound of the deflection.  Defaults: tau = 2e-5,
 * kappa = 3e-7; tau <= 0 disables the FP64 pass.  No counterpart in the
 * reference (which computes everything in FP64). */
int lensgb_model_set_refine(lensgb_model* model, double tau, double kappa);

/* Number of pixels the last image call of this model recomputed in FP64
 * (synchronizes `stream`). */
int lensgb_model_refined_pixels(const lensgb_model* model, void* stream, long long* n);

/* ImageModel.image for n_inst systems (image_model.py:432-492).
 *  params_dev : n_inst x param_count doubles
 *  psf_dev    : PSF kernels, kernel_size^2 values each, FP64 for LENSGB_FP64
 *               and FP32 for LENSGB_FP32_SPLIT, normalised by the caller;
 *               psf_stride = elements between consecutive systems' kernels
 *               (0 = one kernel shared by all systems).  Ignored for
 *               LENSGB_PSF_NONE.
 *  out_dev    : n_inst x ny x nx images, FP64 (LENSGB_FP64) or FP32.
 *  flags      : LENSGB_UNCONVOLVED | LENSGB_NO_SOURCE | LENSGB_NO_LENS_LIGHT */
int lensgb_image(lensgb_model* model, const double* params_dev, int n_inst,
                 const void* psf_dev, long long psf_stride, void* out_dev, int flags,
                 void* stream);

/* lensgb_image with HOST buffers: params_host (n_inst rows), psf_host (as
 * lensgb_image's psf_dev, psf_stride elements apart or shared) and out_host
 * are host memory.  Parameters and PSFs go up and the batch is computed on
 * `stream`, in n_chunks chunks (0: 1); each chunk's images are copied to
 * out_host on a second stream owned by the model, overlapping the next chunk
 * and the next call's work (alternate calls use two device image slots).
 * `stream` does not wait for these copies: lensgb_image_host_wait makes it
 * wait for every copy queued so far (or synchronize the device) before out_host
 * is read.  Page-locked host buffers give the overlap (pageable ones work, with
 * synchronous copies).  Results equal lensgb_image's.  No reference
 * counterpart (the reference returns device arrays that the caller copies). */
int lensgb_image_host(lensgb_model* model, const double* params_host, int n_inst,
                      const void* psf_host, long long psf_stride, void* out_host, int flags,
                      int n_chunks, void* stream);
int lensgb_image_host_wait(lensgb_model* model, void* stream);

/* lensgb_image for systems of different pixel grids in one launch sequence:
 * grids[i] (host) gives system i's grid, PSF size and (optionally)
 * supersampling factor; the model supplies the profile stack, PSF type,
 * precision and the default supersampling (its own grid fields are not used).  psf_dev holds the systems' kernels back to back
 * (kernel_size_i^2 values each), out_dev their images back to back
 * (ny_i x nx_i each).  Each image equals lensgb_image of that system alone,
 * bit for bit.  Not for supersampled convolution or sub-frame models.  The
 * call is asynchronous: its tables go to the device from a page-locked copy
 * owned by the model, and a call waits only until the table copy of the
 * previous call on the same model has run.  No reference counterpart (the
 * reference compiles one program per grid). */
typedef struct {
    int nx, ny;
    double transform_pix2angle[4];
    double ra_at_xy_0, dec_at_xy_0;
    int kernel_size;
    int supersampling;  /* this system's supersampling factor (0: the model's)          */
} lensgb_system_grid;

int lensgb_image_mixed(lensgb_model* model, const double* params_dev, int n_inst,
                       const lensgb_system_grid* grids, const void* psf_dev, void* out_dev,
                       int flags, void* stream);

/* lensgb_image without any device allocation.  No counterpart in the
 * reference: it exists for callers that cannot allocate device memory on the
 * call path -- e.g. a handler invoked from inside an XLA/JAX program (the way a
 * JAX user of the reference would bind this library through jax.ffi), where
 * XLA has already reserved most of the GPU's memory for its own pool, so a
 * cudaMalloc can fail, and cudaFree would synchronize the device under XLA.
 *
 * Same arguments and results as lensgb_image, for every model except two
 * kinds, which it refuses with LENSGB_ERR_UNSUPPORTED (their extra image
 * buffers are not part of the fixed array): models that convolve on the
 * supersampled grid (kwargs_numerics supersampling_convolution=True with
 * s > 1), unless the call passes LENSGB_UNCONVOLVED, which skips that
 * convolution and works; and sub-frame models (lensgb_model_set_subframe,
 * kwargs_numerics flux_evaluate_indexes).  The device scratch (profile
 * records, EPL tables, un-convolved images) comes from a fixed array of
 * LENSGB_NOALLOC_SCRATCH_BYTES inside the library, which every GPU that loads
 * the library holds until exit.  A call whose scratch would exceed it returns
 * LENSGB_ERR_INVALID with the needed size (FP32, 180x180 pixels, EPL+SHEAR and
 * two Sersic profiles: about 267 KB per system, so up to ~250 systems).
 * The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress, with that device current); make that first call
 * before any stream capture.  All calls share the one array: calls that
 * overlap on the GPU race, so issue them on one stream or serialise them.
 * Each call writes every scratch element before reading it, so no state
 * carries over between calls. */
#define LENSGB_NOALLOC_SCRATCH_BYTES (64ull << 20)
int lensgb_image_noalloc(lensgb_model* model, const double* params_dev, int n_inst,
                         const void* psf_dev, long long psf_stride, void* out_dev, int flags,
                         void* stream);

/* PixelKernelConvolution.convolution2d / GaussianConvolution.convolution2d
 * (jaxtronomy/ImSim/Numerics/convolution.py:74-86,215-235) on n_inst images of
 * the model's grid: "same"-mode convolution with the model's PSF type (PIXEL:
 * zero padding, GAUSSIAN: edge padding).  in_dev / out_dev: n_inst x ny x nx in
 * the model precision; psf_dev / psf_stride as for lensgb_image. */
int lensgb_convolve(const lensgb_model* model, const void* in_dev, int n_inst,
                    const void* psf_dev, long long psf_stride, void* out_dev, void* stream);

/* How a model convolves (PIXEL: zero padding; GAUSSIAN: edge padding).  The
 * reference computes jax.scipy.signal.fftconvolve(image, kernel, mode="same")
 * (jaxtronomy/ImSim/Numerics/convolution.py:80-81) or convolve2d (:85); both
 * give the same image up to rounding.  LENSGB_CONV_DIRECT: the shared-memory
 * halo-tile kernels, 2 K^2 flop per pixel.  LENSGB_CONV_FFT: FP64 FFT in shared
 * memory on a P x P grid, P the power of two >= N + K - 1 (plus K - 1 with edge
 * padding, which runs on the explicitly edge-padded image; up to 4096),
 * ~15 P^2 log2(P) flop per image whatever K; its scratch grows with the batch
 * and is allocated on first use.  LENSGB_CONV_AUTO (the default): direct, and
 * the FFT only where the direct kernels' tile does not fit in shared memory
 * (K above ~140 in FP32, ~100 in FP64), so that a model's images keep one
 * summation order in every launch form.  Measured on GB300, direct wins every
 * FP32 case it can run; FP64 models are faster with LENSGB_CONV_FFT from
 * K ~ 21 at 180x180 (3x at K = 41, 11x at K = 85 on 1200x1200). */
#define LENSGB_CONV_AUTO 0
#define LENSGB_CONV_DIRECT 1
#define LENSGB_CONV_FFT 2
int lensgb_model_set_convolution(lensgb_model* model, int method);

/* Halo-tile staging of the FP32 zero-padded convolution (PixelKernelConvolution,
 * jaxtronomy/ImSim/Numerics/convolution.py:74-86, as used by lensgb_image and
 * lensgb_convolve): enable = 1 (the default) fills each CTA's tile with one
 * tensor-memory-accelerator copy where the images allow it (rows a multiple of
 * 16 bytes, 16-byte aligned base, K <= 48), enable = 0 with plain loads.  Both
 * give the same values bit for bit.  Process-wide setting. */
int lensgb_set_conv_tma(int enable);

/* Number of CTAs whose bounded wait for an asynchronous copy gave up (each
 * skips its tile's output) since the library was loaded; 0 in a healthy run.
 * Synchronizes the device. */
int lensgb_wait_timeouts(unsigned int* count);

/* Noise model of the likelihood (ImageData / ImageNoise,
 * jaxtronomy/Data/imaging_data.py:159-182, image_noise.py:16-137).  Strides are
 * elements between consecutive systems; 0 shares one array across systems. */
typedef struct {
    const double* data_dev;       /* ny x nx data per system                      */
    long long data_stride;
    const double* mask_dev;       /* ny x nx likelihood mask (0/1), NULL = all 1   */
    const double* noise_map_dev;  /* ny x nx 1-sigma noise map, NULL = use below   */
    long long noise_stride;
    const double* exposure_map_dev; /* ny x nx exposure map (floored at 1e-10), NULL = scalar */
    long long exposure_stride;
    double exposure_time;         /* scalar exposure (floored at 1e-10)            */
    double background_rms;
    const double* error_map_dev;  /* additional variance map, NULL = none          */
    long long mask_stride;        /* elements between systems' masks (0 = shared)  */
} lensgb_noise_desc;

/* ImageLinearFit's linear amplitude solve (image_linear_solve.py:98-228,
 * 229-341; de_lens.get_param_WLS, de_lens.py:8-38) for n_inst systems of the
 * model's grid: response_dev holds n_linear unit-amplitude component images
 * (component j of system i at (j * n_inst + i) * ny * nx, model precision: the
 * lensgb_image of that component alone with amp = 1).  With the data-based
 * covariance C_D(d) of `noise` (noise map, or max(d, 0)/exposure + bkg^2) and
 * the mask, M = A W A^T and R = A W d are solved for the amplitudes
 * (param_dev, n_inst x n_linear) when cond(M) < 5/eps, else they are 0; the
 * model image sum_j param_j A_j (0 outside the mask) goes to image_out_dev and
 * its log-likelihood (model-based C_D, as lensgb_loglike) to logl_dev.
 * LENSGB_LINEAR_INVERSE (source_marg): M^-1 goes to cov_dev (n_inst x n x n,
 * may be NULL otherwise) and 1/2 log det(M^-1) is added (-1e15 if singular);
 * LENSGB_LINEAR_POSITIVE (check_positive_flux): 1e8 is subtracted when an
 * amplitude is negative.  n_linear <= LENSGB_LINEAR_MAX. */
#define LENSGB_LINEAR_MAX 8
#define LENSGB_LINEAR_INVERSE 1
#define LENSGB_LINEAR_POSITIVE 2
int lensgb_linear_solve(const lensgb_model* model, const void* response_dev, int n_linear,
                        int n_inst, const lensgb_noise_desc* noise, int flags, double* param_dev,
                        double* cov_dev, void* image_out_dev, double* logl_dev, void* stream);

/* ImageModel.likelihood_data_given_model for n_inst systems
 * (image_model.py:163-221): simulates the images into image_out_dev (caller
 * buffer, same layout as lensgb_image's output) and writes one FP64
 * log-likelihood per system to logl_dev. */
/* The likelihood step of lensgb_loglike alone, on given model images (n_inst
 * images in the model precision): Data.log_likelihood (imaging_data.py:159-182)
 * with the model-based C_D (image_noise.py:100-137), e.g. after
 * lensgb_point_sources_add.  FP64 logL per system to logl_dev. */
int lensgb_loglike_image(const lensgb_model* model, const void* image_dev, int n_inst,
                         const lensgb_noise_desc* noise, double* logl_dev, void* stream);

/* ImageModel.point_source (jaxtronomy/ImSim/image_model.py:396-429) ->
 * PointSourceRendering.point_source_rendering
 * (ImSim/Numerics/point_source_rendering.py:34-77): adds to image_dev (n_inst
 * images in the model precision) the point images of each system.  ps_dev:
 * n_inst x n_images x 3 doubles (ra, dec, amp) -- PointSource.point_source_list
 * after ImageModel._displace_astrometry.  kernel_dev: the kernel_size^2 kernel
 * (doubles; the PSF at subgrid factor `subgrid`, or the 3x3 delta of an
 * unconvolved call), kernel_stride doubles apart per system (0: one kernel
 * for all).  Each image is the kernel bilinearly interpolated at the image
 * position on the subgrid (zero outside the kernel, as jax.scipy.ndimage.
 * map_coordinates order 1), summed over each pixel's subgrid^2 cells and
 * scaled by amp and the model's flux_scaling.  Not for sub-frame models. */
int lensgb_point_sources_add(const lensgb_model* model, const double* ps_dev, int n_images,
                             int n_inst, const double* kernel_dev, int kernel_size,
                             long long kernel_stride, int subgrid, void* image_dev, void* stream);

int lensgb_loglike(lensgb_model* model, const double* params_dev, int n_inst,
                   const void* psf_dev, long long psf_stride, const lensgb_noise_desc* noise,
                   void* image_out_dev, double* logl_dev, void* stream);

/* Gradient of ImageModel.likelihood_data_given_model with respect to every
 * column of the system rows -- what jax.grad of the reference's likelihood
 * returns for the kwargs (test_image_model.py:274-335) -- by a hand-written
 * adjoint that recomputes the ray grid.  Same arguments as lensgb_loglike plus
 * grad_dev: n_inst x param_count doubles, row layout.  FP64 models only; lens
 * stacks of EPL, EPL_MULTIPOLE_M1M3M4, SIE, NIE, NFW, TNFW, NFW_ELLIPSE_CSE,
 * CONVERGENCE and SHEAR, SERSIC / SERSIC_ELLIPSE light, at most 64 parameters
 * per row; every PSF type (NONE, PIXEL, GAUSSIAN with its edge padding),
 * convolution on the pixel or on the supersampled grid (with or without a
 * split kernel), and sub-frame models (flux_evaluate_indexes). */
/* Arithmetic of the adjoint's ray derivatives (lensgb_loglike_grad of an FP64
 * model): LENSGB_FP64 (the default) or LENSGB_FP32_SPLIT -- FP32 dual numbers
 * from offsets formed in FP64 per pixel, per-thread sums in FP32 and the
 * reduction over pixels in FP64; the forward image, logL and the weights
 * d logL / d model stay FP64.  Pixels whose rays would lose accuracy in FP32
 * (a predicted relative derivative error above 1e-5, from the source's
 * log-gradient, the distance to its centre and the deflection's size) are
 * recomputed in FP64 by a second pass over those pixels only; measured against
 * the FP64 adjoint the result stays within 1e-4 relative (floor 1e-3 of the
 * largest component).  No counterpart in the reference (jax.grad runs in the
 * precision of the program). */
int lensgb_model_set_grad_precision(lensgb_model* model, int precision);

int lensgb_loglike_grad(lensgb_model* model, const double* params_dev, int n_inst,
                        const void* psf_dev, long long psf_stride, const lensgb_noise_desc* noise,
                        void* image_out_dev, double* logl_dev, double* grad_dev, void* stream);

/* SinglePlane.ray_shooting for one parameter set over n arbitrary points
 * (single_plane.py:39-56), FP64.  params_dev holds the lens profiles' kwargs
 * only (the lens part of a system row). */
int lensgb_ray_shooting(const lensgb_model* model, const double* params_dev,
                        const double* x_dev, const double* y_dev, double* beta_x_dev,
                        double* beta_y_dev, long long n, void* stream);

/* SinglePlane.alpha (single_plane.py:113-139): deflection angles, same
 * arguments as lensgb_ray_shooting. */
int lensgb_alpha(const lensgb_model* model, const double* params_dev, const double* x_dev,
                 const double* y_dev, double* alpha_x_dev, double* alpha_y_dev, long long n,
                 void* stream);

/* LensModel.hessian (jaxtronomy/LensModel/lens_model.py:384-414 ->
 * single_plane.py:142-180) of the model's lens profiles, FP64, for n_inst
 * parameter rows with n points each (x_dev, y_dev: n_inst x n): out_dev
 * receives f_xx, f_xy, f_yx, f_yy as four consecutive arrays of n_inst x n
 * doubles (times alpha_scaling).  EPL, SIE, NIE, NFW, TNFW, SHEAR and
 * CONVERGENCE only (LENSGB_ERR_UNSUPPORTED otherwise). */
int lensgb_hessian(const lensgb_model* model, const double* params_dev, int n_inst,
                   const double* x_dev, const double* y_dev, double* out_dev, long long n,
                   void* stream);

/* LightModel.surface_brightness of the model's source (which = 0) or lens
 * light (which = 1) profiles over n arbitrary points (light_model_base.py:230-252),
 * FP64.  params_dev holds that light model's kwargs only. */
int lensgb_surface_brightness(const lensgb_model* model, int which, const double* params_dev,
                              const double* x_dev, const double* y_dev, double* out_dev,
                              long long n, void* stream);

/* ---- many-deflector ray shooting --------------------------------------- */
/* LensModelBulk(unique_lens_model_list, multi_plane=False)
 * (jaxtronomy/LensModel/lens_model_bulk.py:18-128) -> SinglePlaneBulk
 * (single_plane_bulk.py:20-131).  A bulk handle holds the unique profile
 * codes; each call ray-shoots n points through n_deflectors deflectors:
 *   index_dev   int32[n_deflectors]: position of each deflector's profile in
 *               the unique list; n_unique (or larger) is the NULL profile and
 *               negative values select entry 0, as lax.switch clamps
 *               (the reference's index_list, single_plane_bulk.py:93-95)
 *   params_dev  double[n_deflectors][LENSGB_BULK_PARAM_STRIDE]: each
 *               deflector's kwargs in its profile's param_names order (the
 *               table at the top), unused columns ignored (the reference's
 *               all_kwargs dict of arrays, single_plane_bulk.py:97-106)
 *   beta = x - sum_i alpha_i(x)               (single_plane_bulk.py:128-131)
 * Precision LENSGB_FP64 evaluates every term in FP64.  LENSGB_FP32_SPLIT
 * evaluates a deflector's terms in FP32 when its deflection is bounded by
 * fp32_alpha_max (|alpha| <= theta_E for SIE/NIE/EPL/EPL_MULTIPOLE_M1M3M4,
 * <= 2 alpha_Rs for NFW/TNFW/NFW_ELLIPSE_CSE; SHEAR never), sums those terms
 * in FP32 over chunks of 64 deflectors and accumulates the chunk sums, and
 * every FP64 term, in FP64.  The handle owns grow-only device scratch
 * (about 340 B per deflector, plus 6 KB per deflector when an EPL-type or
 * NFW_ELLIPSE_CSE profile is in the unique list) and serves one stream at a
 * time. */
#define LENSGB_LENS_NULL 0 /* the reference's "NULL" profile: no deflection */
#define LENSGB_BULK_MAX_UNIQUE 16
#define LENSGB_BULK_PARAM_STRIDE 12

typedef struct lensgb_bulk lensgb_bulk;

int lensgb_bulk_create(const int* unique_codes, int n_unique, int precision,
                       lensgb_bulk** out);
int lensgb_bulk_destroy(lensgb_bulk* bulk);
/* Largest deflection bound (arcsec) evaluated in FP32 (default 0.05). */
int lensgb_bulk_set_fp32_alpha_max(lensgb_bulk* bulk, double alpha_max);
int lensgb_bulk_ray_shooting(lensgb_bulk* bulk, const int* index_dev, const double* params_dev,
                             int n_deflectors, const double* x_dev, const double* y_dev,
                             double* beta_x_dev, double* beta_y_dev, long long n, void* stream);

/* LensModelBulk(unique_lens_model_list, multi_plane=True) -> MultiPlaneBulk
 * (jaxtronomy/LensModel/MultiPlane/multi_plane_bulk.py:11-272):
 * ray_shooting(alpha_x, alpha_y, all_kwargs, index_list, T_ij_list, T_z_list,
 * reduced2physical_factor) (:152-200).  The n_steps steps are the
 * redshift-sorted deflectors, the source plane and the NULL fillers that
 * prepare_ray_shooting_kwargs builds (:57-150), with index_dev / params_dev as
 * in lensgb_bulk_ray_shooting and, per step, T_ij_dev (transverse comoving
 * distance from the previous step), T_z_dev (from the observer) and r2p_dev
 * (reduced-to-physical deflection factor).  Starting from x = 0 at angles
 * alpha (arcsec), every step does x += alpha T_ij; alpha -= r2p *
 * alpha_i(x / T_z); beta = x / T_z[n_steps - 1].  n_steps >= 1.
 * LENSGB_FP64 follows that recurrence in FP64.  LENSGB_FP32_SPLIT carries the
 * deflection and displacement as FP32 pairs next to the FP64 start angle,
 * groups consecutive deflectors of one plane (T_ij = 0, equal T_z and r2p),
 * evaluates fp32_alpha_max-bounded terms in FP32, CONVERGENCE as an FP32-pair
 * product and the other terms in FP64. */
int lensgb_bulk_multi_plane_ray_shooting(lensgb_bulk* bulk, const int* index_dev,
                                         const double* params_dev, int n_steps,
                                         const double* T_ij_dev, const double* T_z_dev,
                                         const double* r2p_dev, const double* alpha_x_dev,
                                         const double* alpha_y_dev, double* beta_x_dev,
                                         double* beta_y_dev, long long n, void* stream);

/* ---- serving loop ---------------------------------------------------------- */
/* A server batches independent image / likelihood requests continuously: a
 * worker thread groups released requests by bucket (identical
 * lensgb_model_desc and noise options), keeps up to n_streams batches in
 * flight on separate CUDA streams -- requests arriving while others run join
 * the next batch of their bucket as soon as a stream is free -- and stages
 * each request's parameters, PSF, data, noise map and mask in device buffers
 * of a per-bucket execution context.  The device memory of all contexts is
 * kept under hbm_budget_bytes by evicting idle contexts (least recently used
 * first); requests wait in their queue while batches in flight hold the
 * budget.  With use_graphs, a batch size that a context has run once is
 * captured as a CUDA graph and replayed.  Each request's result is the same as
 * a lensgb_image / lensgb_loglike call on that request alone (the kernels
 * compute every system independently of the others in its batch).
 * No counterpart in the reference, which simulates one jitted call at a time. */
typedef struct lensgb_server lensgb_server;

typedef struct {
    int n_streams;              /* batches in flight at once (default 4, <= 64)        */
    int max_batch;              /* requests per batch (default 256)                    */
    long long hbm_budget_bytes; /* device memory of all contexts (default 4 GiB)       */
    int contexts_per_bucket;    /* concurrent batches of one bucket (default 2)        */
    int use_graphs;             /* replay captured CUDA graphs for repeated sizes      */
    int mixed_grids;            /* 1: image requests whose models differ only in the
                                   grid (nx, ny, transform_pix2angle, ra/dec_at_xy_0)
                                   and kernel_size share a bucket, whose batches run
                                   through lensgb_image_mixed; 2: also requests of
                                   different supersampling factors (one ray-kernel
                                   launch per factor in each batch); likelihood and
                                   supersampled-convolution requests keep exact-model
                                   buckets                                             */
} lensgb_server_config;

/* One serving request.  psf, data, noise_map, mask and image_out may be host
 * memory (pageable: staged through page-locked buffers; page-locked: read and
 * written by the device in place) or memory of the server's device, which
 * stays resident across requests -- the form of ImageData.update_data /
 * ImageNoise.C_D_model keeping a model's data on the device
 * (jaxtronomy/Data/imaging_data.py:135-157, image_noise.py:100-110): the gather
 * kernels read it where it is, with no host copy per batch.  A request whose
 * PSF is in device memory runs in an exact-model bucket. */
typedef struct {
    lensgb_model_desc desc;     /* the request's model (its bucket key)                    */
    const double* params;       /* host: lensgb_model_param_count doubles (one system row) */
    const void* psf;            /* kernel_size^2 values in the model precision             */
    void* image_out;            /* ny x nx result in the model precision, or NULL;
                                   page-locked / device buffers are written by the device  */
    const double* data;         /* optional: ny x nx data -> likelihood request            */
    const double* noise_map;    /* optional with data: ny x nx 1-sigma noise map           */
    const double* mask;         /* optional with data: ny x nx likelihood mask             */
    double background_rms;      /* with data (part of the bucket key)                      */
    double exposure_time;       /* with data (part of the bucket key)                      */
    double* logl_out;           /* host, optional with data: log-likelihood                */
    long long release_ns;       /* not admitted before this server-clock time (0: now)     */
} lensgb_request;

#define LENSGB_REQ_QUEUED 0
#define LENSGB_REQ_RUNNING 1
#define LENSGB_REQ_DONE 2
#define LENSGB_REQ_FAILED 3
#define LENSGB_REQ_CANCELLED 4

typedef struct {
    long long batches;
    long long requests_launched;
    long long requests_done;
    long long graph_captures;
    long long graph_launches;
    long long evictions;
    long long bytes_held;
    long long peak_bytes;
    long long host_launch_ns;   /* worker time spent staging and launching batches */
    long long capture_ns;       /* of which capturing and instantiating graphs      */
    long long mixed_batches;    /* batches run through lensgb_image_mixed           */
} lensgb_server_stats;

/* cfg may be NULL (defaults); zero fields take their defaults.  The server
 * runs on the device current on the calling thread. */
int lensgb_server_create(const lensgb_server_config* cfg, lensgb_server** out);
/* Queues n requests (the host buffers they name must stay valid until each is
 * done); tickets[i] receives request i's ticket.  Validates each request's
 * model; on an error no later request of the call is queued. */
int lensgb_server_submit(lensgb_server* server, const lensgb_request* requests, int n,
                         long long* tickets);
/* *state = LENSGB_REQ_*; returns the request's error code once it FAILED. */
int lensgb_server_poll(lensgb_server* server, long long ticket, int* state);
/* Withdraws a request that has not been admitted to a batch yet: *cancelled = 1
 * and the request ends in state LENSGB_REQ_CANCELLED (it never runs and its
 * buffers are not touched again); *cancelled = 0 when it is already running or
 * finished.  A request the server cannot fit in hbm_budget_bytes even with
 * every idle context evicted and nothing in flight ends FAILED with
 * LENSGB_ERR_OOM. */
int lensgb_server_cancel(lensgb_server* server, long long ticket, int* cancelled);
/* Polls until the request is done, failed or cancelled, or timeout_s elapses
 * (then returns LENSGB_OK with the state it has). */
int lensgb_server_wait(lensgb_server* server, long long ticket, double timeout_s, int* state);
/* Waits until every submitted request is done or failed. */
int lensgb_server_drain(lensgb_server* server, double timeout_s);
/* Server clock (ns since creation), the time base of release_ns. */
long long lensgb_server_clock_ns(const lensgb_server* server);
/* Release, admission and completion times of a request (-1 while not reached). */
int lensgb_server_request_times(lensgb_server* server, long long ticket, long long* release_ns,
                                long long* admit_ns, long long* done_ns);
int lensgb_server_get_stats(lensgb_server* server, lensgb_server_stats* out);
/* Finishes the batches in flight, then frees everything; queued requests that
 * were never launched stay QUEUED. */
int lensgb_server_destroy(lensgb_server* server);

/* Description of the last error on the calling thread ("" if none). */
const char* lensgb_last_error(void);

/* FMA-rate probe.  No counterpart in the reference: it measures the device's
 * FP32 (precision LENSGB_FP32_SPLIT), FP64 (LENSGB_FP64) or packed-pair FP32
 * (LENSGB_FP32_PAIRS: fma.rn.f32x2, two FMAs per instruction) fused
 * multiply-add rate, the peak against which the roofline fractions of the
 * compute-bound kernels are stated.  Launches `blocks` CTAs of 256 threads, each running 8
 * independent chains of `iters` FMAs (iters a multiple of 16), and writes one
 * value per thread to out_dev (blocks x 256 elements of that precision).
 * *flops receives the launch's flop count (2 per FMA); time the launch with
 * events on `stream`. */
#define LENSGB_FP32_PAIRS 2
int lensgb_fma_chain(int precision, int blocks, int iters, void* out_dev, long long* flops,
                     void* stream);

/* ABI version of this header (major * 100 + minor). */
int lensgb_version(void);

#ifdef __cplusplus
}
#endif
#endif /* LENSGB_H */
