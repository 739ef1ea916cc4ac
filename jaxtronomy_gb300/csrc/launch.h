// Host-side launchers shared between the kernel translation units and the
// C ABI (abi.cu).  Internal to liblensgb.so.
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

#include <string>

namespace lensgb {

// Sets the calling thread's lensgb_last_error() text (defined in abi.cu).
void set_last_error(const std::string& msg);

// Streaming multiprocessors of the current device (launch shapes), read from
// the device once per device.
inline int num_sms() {
    static int cached[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    if (cached[dev] <= 0) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            n <= 0) {
            cudaGetLastError();
            n = 1;
        }
        cached[dev] = n;
    }
    return cached[dev];
}

// Per-system profile records of n_inst systems (grids: per-system grids of a
// mixed launch; n_dev: device count of systems actually present, <= n_inst).
int launch_prepare(const GridDesc& g, const StackDesc& st, const double* params, int n_inst,
                   double* rec_d, float* rec_f, double* coef_d, float* coef_f,
                   cudaStream_t stream, const GridDesc* grids = nullptr,
                   const int* n_dev = nullptr);

// Supersampled ray tracing + light + s x s re-binning into a (ny, nx) image per
// system, scaled by out_scale (pixel_width^2).  `precision` selects FP64 or FP32;
// the FP32 path refines flagged pixels in FP64 as described by `rf`
// (rf.count must be zero on the stream when the launch starts).
// `mixed` (device tables, or null): systems of different grids in one launch
// of mixed_ctas CTAs looping over the systems' tiles (g then only supplies s);
// images are laid out at mixed->off.
// ppt > 0 (uniform launches): pixels per thread instead of the built-in choice.
int launch_raytrace(const GridDesc& g, const StackDesc& st, int n_inst, const double* rec_d,
                    const float* rec_f, const double* coef_d, const float* coef_f, void* out,
                    int flags, double out_scale, int precision, const RefineArgs& rf,
                    cudaStream_t stream, const MixedTab* mixed = nullptr, int mixed_ctas = 0,
                    int ppt = 0);

// "same"-mode convolution by FP64 FFT (fftconv.cu), zero (edge = 0) or edge
// padding (edge = 1): P (a power of two >= max(ny, nx) + K - 1, plus K - 1 with
// edge padding; at most 4096) and the scratch it needs; returns 0, -1
// (shared-memory configuration) or -2 (P above 4096).
int fft_conv_size(int ny, int nx, int K, int edge);
size_t fft_conv_scratch_bytes(int n_inst, int ny, int nx, int K, long long kstride, int edge);
int launch_conv_fft(const void* in, void* out, const void* kernel, long long kstride, int n_inst,
                    int ny, int nx, int K, int edge, int precision, void* scratch,
                    cudaStream_t stream);
// Whether the direct kernels' shared-memory tile fits for a K x K kernel.
bool direct_conv_fits(int K, int precision);

// FP32 zero-padded uniform convolutions stage their halo tiles with a TMA copy
// when the images allow it (set_conv_tma(0): plain loads everywhere);
// conv_wait_timeouts: CTAs whose bounded wait for that copy gave up (synchronous).
void set_conv_tma(int enable);
unsigned int conv_wait_timeouts();

// "same"-mode 2-D convolution of n_inst (ny, nx) images with K x K kernels
// (kernel stride 0 = shared).  edge = 0: zero padding; 1: edge padding.
// tile_rows (FP32; a multiple of 4 in 32..64, 0: the built-in choice): output
// rows per CTA tile.
int launch_conv(const void* in, void* out, const void* kernel, long long kstride, int n_inst,
                int ny, int nx, int K, int edge, int precision, cudaStream_t stream,
                int tile_rows = 0);

// Convolution of systems of different sizes (tables in `cm`): one launch of
// n_ctas CTAs looping over the tiles of the group's systems, whose kernels are
// at most kmax wide; FP32 `group` g > 0 runs the kernel specialised for widths
// <= 8 g (systems are grouped by it), 0 the run-time-width one.  Tiles are
// 64 x 64 (FP32) / 32 x 64 (FP64) pixels.
int launch_conv_mixed(const void* in, void* out, const void* kernel, const ConvMixed& cm,
                      int n_ctas, int kmax, int group, int edge, int precision,
                      cudaStream_t stream);

// ---- mixed-grid launches (abi.cu) -------------------------------------------
// Offsets, in one device / page-locked table block, of the per-system tables
// of a mixed launch for up to `cap` systems (see MixedTab / ConvMixed).
struct MixedLayout {
    int cap;
    size_t o_n, o_grid, o_off, o_koff, o_ks, o_scale;
    size_t o_rsys, o_rtoff, o_rcnt;  // ray groups: systems, tile prefix, counts
    size_t o_gsys, o_goff, o_gcnt;   // convolution groups: the same
    size_t bytes;
};
MixedLayout mixed_layout(int cap);

// Ray-kernel groups: FP32 s = 1..4 (compile-time s), 0 every other s; FP64
// uses group 0 only.  Convolution groups: index 0 for FP64, 1..6 the
// fixed-width FP32 kernels, 7 the run-time-width FP32 kernel.
constexpr int MIX_RAY_GROUPS = 5;
constexpr int MIX_CONV_GROUPS = 8;

// Host-side totals of a filled table block.
struct MixedCounts {
    int n;
    long long pix, kel;
    int ray_tiles[MIX_RAY_GROUPS];
    int conv_tiles[MIX_CONV_GROUPS];
    int kmax[MIX_CONV_GROUPS];
};

// Launch configuration: CTAs of each ray group and of each convolution group
// (0: the group is not launched) and the widest kernel each convolution group
// may meet.
struct MixedGrid {
    int ray_ctas[MIX_RAY_GROUPS];
    int conv_ctas[MIX_CONV_GROUPS];
    int conv_kmax[MIX_CONV_GROUPS];
};

// Validates n system grids and writes their tables into host block H.
int mixed_fill(const lensgb_model* m, unsigned char* H, const MixedLayout& L,
               const lensgb_system_grid* grids, int n, bool conv, MixedCounts* out);
// Grows the model's scratch for cap systems of `pix` pixels in total.
int mixed_reserve(lensgb_model* m, int cap, long long pix, size_t table_bytes);
// Stream operations of one mixed launch over at most n_cap systems whose tables
// are at device address tab (the system count is read on the device): records,
// ray tracing (+ FP32 refinement), grouped convolution.  Allocates nothing, so
// it can be captured into a CUDA graph after mixed_reserve.
int mixed_launch(lensgb_model* m, const double* params_dev, int n_cap, const unsigned char* tab,
                 const MixedLayout& L, const MixedGrid& gr, const void* psf, void* out, int flags,
                 cudaStream_t st);

// s x s block mean (image_util.re_size, image_util.py:79-98: mean over
// sub-columns, then sub-rows) of n_inst (ny*s, nx*s) images, times scale.
int launch_resize(const void* hr, void* out, int n_inst, int ny, int nx, int s, double scale,
                  int precision, cudaStream_t stream);

// Multiply n_inst (ny*s, nx*s) images by an (ny, nx) 0/1 mask (mask[r/s][c/s]).
int launch_mask(void* img, int n_inst, int ny, int nx, int s, const unsigned char* mask,
                int precision, cudaStream_t stream);
// out (n_inst full ny_full x nx_full images) = 0 except the n x n block at
// (r0, c0), which receives `sub`.
int launch_embed(const void* sub, void* out, int n_inst, int n, int r0, int c0, int ny_full,
                 int nx_full, int precision, cudaStream_t stream);

// out[i] = (out[i] + add[i]) * scale over n elements.
int launch_add_scaled(void* out, const void* add, long long n, double scale, int precision,
                      cudaStream_t stream);

// Noise description of the likelihood reduction (device pointers; strides in
// elements between systems, 0 = shared by all systems).
struct LoglikeArgs {
    const double* data;
    long long data_stride;
    const double* mask;       // ny*nx per system (mask_stride apart) or null (all pixels)
    long long mask_stride;
    const double* noise_map;  // or null
    long long noise_stride;
    const double* exposure;   // exposure map (already floored) or null
    long long exposure_stride;
    double exposure_time;     // used when exposure is null
    double background_rms;
    const double* error_map;  // additional variance map or null
};

int launch_loglike(const void* model, int n_inst, long long npix, const LoglikeArgs& a,
                   double* out, int precision, cudaStream_t stream);

// Linear amplitude solve (linear.cu): see lensgb_linear_solve.
constexpr int LIN_MAX = LENSGB_LINEAR_MAX;
int launch_linear_solve(const void* A, int n_lin, int n_inst, long long npix, const LoglikeArgs& a,
                        int flags, double* param, double* cov, void* image, double* logl,
                        int precision, cudaStream_t stream);

// Adjoint gradient of logL (grad.cu), FP64, in stages that lensgb_loglike_grad
// chains (the reverse of the forward image path):
//   launch_grad_weights: logL and g_m = d logL / d model per pixel;
//   launch_crop: the sub-frame of a full-frame array (sub-frame models);
//   launch_conv_transpose: the transposed "same" convolution (the PSF rotated
//     by 180 degrees; edge = 1: edge padding, through pad_a / pad_b scratch of
//     (ny + K - 1) x (nx + K - 1) per system); psf_flip: n_inst x K^2 scratch;
//   launch_expand: the transposed s x s block mean (hr = low x scale per block);
//   launch_grad_rays: forward-mode derivatives (precision LENSGB_FP64, or
//     LENSGB_FP32_SPLIT: FP32 dual numbers from FP64-accurate offsets, pixels
//     predicted ill-conditioned recomputed in FP64; `flag`: n_inst x pixels of g
//     bytes, `partial` then twice its FP64 size) of every ray of grid g weighted
//     by gl x w_scale / s^2 x flux_scaling, summed per parameter in a fixed
//     order into grad (n_inst x n_params); dcoef: n_inst x n_epl x EPL_NMAX and
//     partial: n_inst x grad_chunks(g) x n_params scratch.
// grad_supported: every lens profile has a Jacobian (EPL, EPL_MULTIPOLE_M1M3M4,
// SIE, NIE, NFW, TNFW, NFW_ELLIPSE_CSE, CONVERGENCE, SHEAR) and the row has at
// most 64 parameters.
bool grad_supported(const StackDesc& st);
int grad_chunks(const GridDesc& g);
int launch_grad_weights(const double* image, int n_inst, long long npix, const LoglikeArgs& la,
                        double* gm, double* logl, cudaStream_t stream);
int launch_crop(const double* full, double* sub, int n_inst, int n, int r0, int c0, int ny_full,
                int nx_full, cudaStream_t stream);
int launch_conv_transpose(const double* in, double* out, const double* psf, long long psf_stride,
                          int K, int edge, int n_inst, int ny, int nx, double* psf_flip,
                          double* pad_a, double* pad_b, cudaStream_t stream);
int launch_expand(const double* low, double* hr, int n_inst, int ny, int nx, int s, double scale,
                  int accumulate, cudaStream_t stream);
int launch_scale(double* x, long long n, double a, cudaStream_t stream);
int launch_grad_rays(const GridDesc& g, const StackDesc& st, int n_inst, const double* params,
                     const double* rec_d, const double* coef_d, double* dcoef, const double* gl,
                     double w_scale, double* partial, double* grad, int precision,
                     unsigned char* flag, float tau, cudaStream_t stream);

// Point-wise single-parameter-set evaluation (FP64).
int launch_ray_shoot_points(const StackDesc& st, const double* rec_d, const double* coef_d,
                            const double* x, const double* y, double* bx, double* by,
                            long long n, int want_alpha, cudaStream_t stream);
int launch_light_points(const StackDesc& st, int which, const double* rec_d, const double* x,
                        const double* y, double* out, long long n, cudaStream_t stream);

// Many-deflector ray shooting (LensModelBulk).  The prepare step turns
// n_defl kwargs rows (LENSGB_BULK_PARAM_STRIDE doubles each) into records and
// tags; coef_d/coef_f hold EPL_NMAX entries per deflector (or are null when
// no unique profile needs a coefficient table).
int launch_bulk_prepare(const BulkUnique& u, const int* index, const double* params, int n_defl,
                        double fp32_alpha_max, int* tag, double* rec_d, float* rec_f,
                        double* coef_d, float* coef_f, cudaStream_t stream);
// beta = x - sum_i alpha_i(x) over n rays.  precision FP64: every term in
// FP64; FP32_SPLIT: deflectors without BULK_TAG_FP64 run in FP32, summed in
// FP32 per chunk of deflectors and accumulated in FP64.
int launch_bulk_ray_shooting(const int* tag, const double* rec_d, const float* rec_f,
                             const double* coef_d, const float* coef_f, int n_defl,
                             const double* x, const double* y, double* bx, double* by,
                             long long n, int precision, cudaStream_t stream);
// LensModel.hessian at n points (out: f_xx, f_xy, f_yx, f_yy, n each) from the
// lens records of one parameter row; hessian_supported: every lens profile has
// position derivatives (EPL, EPL_MULTIPOLE_M1M3M4, SIE, NIE, NFW, TNFW,
// NFW_ELLIPSE_CSE, SHEAR, CONVERGENCE).
bool hessian_supported(const StackDesc& st);
int launch_hessian_points(const StackDesc& st, const double* rec, const double* coef,
                          const double* params, const double* x, const double* y, double* out,
                          long long n, long long n_per, cudaStream_t stream);
// Point-source rendering: adds to out (n_inst images of rows x cols, model
// precision) the n_img images (ra, dec, amp) of each system, the kernel
// (ks x ks doubles; kstride per system, 0: shared) at subgrid factor p.
int launch_point_sources(const double* ps, int n_img, int n_inst, const double* K, int ks,
                         long long kstride, int p, const double* Ma2pix, double x0, double y0,
                         int rows, int cols, double scale, void* out, int precision,
                         cudaStream_t stream);
// MultiPlaneBulk.ray_shooting over n_steps redshift-ordered steps (tags and
// records from launch_bulk_prepare; T_ij, T_z, r2p per step) for n rays
// starting at angles (ax, ay).  FP32_SPLIT also writes the plane table pl_f
// (8 floats per step), eps_d (n_steps doubles) and the tags' plane flags.
int launch_multi_plane(int* tag, const double* rec_d, const float* rec_f, const double* coef_d,
                       const float* coef_f, float* pl_f, double* eps_d, const double* dT,
                       const double* Tz, const double* r2p, int n_steps, const double* ax,
                       const double* ay, double* bx, double* by, long long n, int precision,
                       cudaStream_t stream);

}  // namespace lensgb
