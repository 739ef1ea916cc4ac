// C ABI of liblensgb.so (declared in include/lensgb.h).
//
// A model handle is the compiled form of one ImageModel
// (JAXtronomy ImSim/image_model.py:27-150): the profile stack, the pixel grid
// and numerics options, plus grow-only device scratch for the per-profile
// records, the EPL coefficient tables and the un-convolved image.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "launch.h"

using namespace lensgb;

struct lensgb_model {
    lensgb_model_desc desc;
    GridDesc grid;
    GridDesc grid_hr;            // the supersampled grid as a grid of its own (s = 1)
    bool hr_conv = false;        // convolution on the supersampled grid
    void* hr_img = nullptr;      // supersampled image and its convolution (hr_conv models)
    void* hr_out = nullptr;
    // sub-frame (NumericsSubFrame): the kernels run on `grid`, an n x n sub-frame
    // whose images are embedded at (sub_r0, sub_c0) of the full image
    bool sub = false;
    int sub_r0 = 0, sub_c0 = 0;
    unsigned char* sub_mask = nullptr;  // n x n evaluation mask (device), or null
    void* sub_out = nullptr;            // sub-frame images before embedding
    // lensgb_image_mixed scratch (grow-only): tables and per-pixel buffers
    size_t mix_tab_cap = 0, mix_pix_cap = 0;
    unsigned char* mix_tab = nullptr;
    void* mix_low = nullptr;
    unsigned int* mix_list = nullptr;
    // page-locked host copy of the tables; mix_ev marks the end of the last
    // table copy, before which the host buffer is not rewritten
    size_t mix_host_cap = 0;
    unsigned char* mix_host = nullptr;
    // lensgb_image_host: device staging (grow-only; two image slots used by
    // alternate calls, so a call's image copies overlap the next call's work),
    // the copy-back stream, one event per chunk and one per slot
    size_t pipe_rows_cap = 0, pipe_psf_cap = 0, pipe_out_cap[2] = {0, 0};
    void* pipe_rows = nullptr;
    void* pipe_psf = nullptr;
    void* pipe_out[2] = {nullptr, nullptr};
    int pipe_slot = 0;
    cudaStream_t pipe_stream = nullptr;
    cudaEvent_t pipe_ev[16] = {};
    cudaEvent_t pipe_slot_ev[2] = {};
    cudaEvent_t pipe_wait_ev = nullptr;
    cudaEvent_t mix_ev = nullptr;
    bool mix_ev_pending = false;
    StackDesc st;
    double pixel_width;
    int cap_inst = 0;
    double* rec_d = nullptr;
    float* rec_f = nullptr;
    double* coef_d = nullptr;
    float* coef_f = nullptr;
    void* lowres = nullptr;
    unsigned int* refine_list = nullptr;  // FP32 models: one entry per pixel
    unsigned int* refine_count = nullptr;
    float refine_tau = 2e-5f;             // see lensgb_model_set_refine
    int tune_ppt = 0, tune_rows = 0;      // launch shapes (lensgb_model_autotune; 0: built-in)
    long long tune_pix = 0;               // pixels of the tuned call; tuned ppt applies from 1/4 of it
    float refine_kappa = 3e-7f;
    // convolution method (lensgb_model_set_convolution) and the FFT path's scratch
    int conv_method = LENSGB_CONV_AUTO;
    int grad_precision = LENSGB_FP64;  // lensgb_model_set_grad_precision
    void* fft_scratch = nullptr;
    size_t fft_cap = 0;
    // gradient scratch (lensgb_loglike_grad), grow-only
    int grad_cap = 0;
    double* g_dcoef = nullptr;
    double* g_psf = nullptr;      // flipped kernels (pixel-scale or supersampled, then low-res)
    double* g_m = nullptr;        // d logL / d model, full frame
    double* g_a = nullptr;        // kernel-grid arrays (sub-frame crop, transposed convolution)
    double* g_b = nullptr;
    double* g_c = nullptr;        // supersampled-grid arrays (supersampled convolution)
    double* g_d = nullptr;
    double* g_pad_a = nullptr;    // edge-padded arrays (GAUSSIAN transposed convolution)
    double* g_pad_b = nullptr;
    double* g_partial = nullptr;
    double* g_flag = nullptr;     // FP32 adjoint: one byte per ray-grid pixel (flagged for FP64)
    float grad_tau = 1e-5f;       // FP32 adjoint: predicted relative error that flags a pixel
};

static void free_grad_scratch(lensgb_model* m) {
    double** bufs[] = {&m->g_dcoef, &m->g_psf, &m->g_m, &m->g_a, &m->g_b,
                       &m->g_c, &m->g_d, &m->g_pad_a, &m->g_pad_b, &m->g_partial,
                       &m->g_flag};
    for (double** b : bufs) {
        cudaFree(*b);
        *b = nullptr;
    }
    m->grad_cap = 0;
}

static thread_local std::string g_last_error;

static int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

void lensgb::set_last_error(const std::string& msg) { g_last_error = msg; }

static int lens_param_count(int code) {
    switch (code) {
        case LENSGB_LENS_SIE: return 5;
        case LENSGB_LENS_NIE: return 6;
        case LENSGB_LENS_EPL: return 6;
        case LENSGB_LENS_SHEAR: return 4;
        case LENSGB_LENS_NFW: return 4;
        case LENSGB_LENS_TNFW: return 5;
        case LENSGB_LENS_NFW_ELLIPSE_CSE: return 6;
        case LENSGB_LENS_CONVERGENCE: return 3;
        case LENSGB_LENS_EPL_MULTIPOLE_M1M3M4: return 12;
        default: return -1;
    }
}

static int light_param_count(int code) {
    switch (code) {
        case LENSGB_LIGHT_SERSIC: return 5;
        case LENSGB_LIGHT_SERSIC_ELLIPSE: return 7;
        default: return -1;
    }
}

static int check_cuda(const char* where) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return fail(LENSGB_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
    return LENSGB_OK;
}

static void free_scratch(lensgb_model* m) {
    cudaFree(m->rec_d);
    cudaFree(m->rec_f);
    cudaFree(m->coef_d);
    cudaFree(m->coef_f);
    cudaFree(m->lowres);
    cudaFree(m->refine_list);
    cudaFree(m->refine_count);
    cudaFree(m->hr_img);
    cudaFree(m->hr_out);
    cudaFree(m->sub_out);
    m->hr_img = nullptr;
    m->hr_out = nullptr;
    m->sub_out = nullptr;
    m->refine_list = nullptr;
    m->refine_count = nullptr;
    m->rec_d = nullptr;
    m->rec_f = nullptr;
    m->coef_d = nullptr;
    m->coef_f = nullptr;
    m->lowres = nullptr;
    m->cap_inst = 0;
}

static int ensure_scratch(lensgb_model* m, int n_inst) {
    if (n_inst <= m->cap_inst) return LENSGB_OK;
    int cap = m->cap_inst > 0 ? m->cap_inst : 1;
    while (cap < n_inst) cap *= 2;
    free_scratch(m);
    const int n_prof = m->st.n_lens + m->st.n_src + m->st.n_ll;
    const size_t nrec = (size_t)cap * (n_prof > 0 ? n_prof : 1);
    const size_t ncoef = (size_t)cap * (m->st.n_epl > 0 ? m->st.n_epl : 1) * EPL_NMAX;
    const size_t esz = m->desc.precision == LENSGB_FP64 ? 8 : 4;
    const size_t nimg = (size_t)cap * m->grid.nx * m->grid.ny;
    const size_t s2 = (size_t)m->grid.s * m->grid.s;
    // refine list: one entry per ray of the grid the FP32 kernel runs on
    const size_t nlist = m->hr_conv ? nimg * s2 : nimg;
    if (cudaMalloc(&m->rec_d, nrec * REC_D * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&m->rec_f, nrec * REC_F * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&m->coef_d, ncoef * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&m->coef_f, ncoef * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&m->lowres, nimg * esz) != cudaSuccess ||
        (m->desc.precision == LENSGB_FP32_SPLIT &&
         (cudaMalloc(&m->refine_list, nlist * sizeof(unsigned int)) != cudaSuccess ||
          cudaMalloc(&m->refine_count, sizeof(unsigned int)) != cudaSuccess)) ||
        (m->hr_conv && (cudaMalloc(&m->hr_img, nimg * s2 * esz) != cudaSuccess ||
                        cudaMalloc(&m->hr_out, nimg * s2 * esz) != cudaSuccess)) ||
        (m->sub && cudaMalloc(&m->sub_out, nimg * esz) != cudaSuccess)) {
        cudaGetLastError();
        free_scratch(m);
        return fail(LENSGB_ERR_OOM, "device allocation of model scratch failed");
    }
    m->cap_inst = cap;
    return LENSGB_OK;
}

// Number of significant bits of the FP32 "exact" step so that index * step
// stays exact for every supersampled index of the grid.
static int exact_bits(int n) {
    int b = 0;
    while ((1 << b) < n) ++b;
    int bits = 24 - b;
    return bits < 1 ? 1 : bits;
}

// Refinement of the FP32 path: active for FP32 models with tau > 0, when the
// global pixel index of the batch fits the 32-bit list entries.
static RefineArgs refine_args(const lensgb_model* m, int n_inst, unsigned int* list,
                              unsigned int* count) {
    RefineArgs rf;
    rf.list = list;
    rf.count = count;
    rf.kappa = m->refine_kappa;
    rf.tau = 0.f;
    if (m->desc.precision == LENSGB_FP32_SPLIT && m->refine_tau > 0.f && list && count)
        rf.tau = m->refine_tau;
    return rf;
}

// The refine list stores 32-bit batch-global pixel indices.
// Kernel grids of an nx x ny pixel grid whose pixel (0, 0) is at (ra0, dec0),
// with the model's transform and supersampling: the image grid and its
// supersampled twin (s = 1), as the ray kernels index them.
static GridDesc make_grid(int nx, int ny, int s, const double* M, double ra0, double dec0) {
    GridDesc g;
    g.nx = nx;
    g.ny = ny;
    g.s = s;
    const double f0 = 0.5 / s - 0.5;
    g.ra00 = ra0 + M[0] * f0 + M[1] * f0;
    g.dec00 = dec0 + M[2] * f0 + M[3] * f0;
    g.ax = M[0] / s;
    g.bx = M[1] / s;
    g.ay = M[2] / s;
    g.by = M[3] / s;
    const int bits = exact_bits((nx > ny ? nx : ny) * s);
    split_bits(g.ax, bits, g.ax_hi, g.ax_lo);
    split_bits(g.bx, bits, g.bx_hi, g.bx_lo);
    split_bits(g.ay, bits, g.ay_hi, g.ay_lo);
    split_bits(g.by, bits, g.by_hi, g.by_lo);
    return g;
}

static void set_grids(lensgb_model* m, int nx, int ny, double ra0, double dec0) {
    const lensgb_model_desc* d = &m->desc;
    m->grid = make_grid(nx, ny, d->supersampling, d->transform_pix2angle, ra0, dec0);
    const GridDesc& g = m->grid;
    const int s = d->supersampling;
    m->grid_hr = g;
    m->grid_hr.nx = g.nx * s;
    m->grid_hr.ny = g.ny * s;
    m->grid_hr.s = 1;
}

static int check_refine_size(const lensgb_model* m, int n_inst) {
    const long long s2 = m->hr_conv ? (long long)m->grid.s * m->grid.s : 1;
    if (m->desc.precision == LENSGB_FP32_SPLIT && m->refine_tau > 0.f &&
        (long long)n_inst * m->grid.nx * m->grid.ny * s2 >= (1LL << 32))
        return fail(LENSGB_ERR_INVALID,
                    "n_inst * nx * ny must stay below 2^32 for FP32 models; split the batch");
    return LENSGB_OK;
}

extern "C" {

int lensgb_version(void) { return 116; }

int lensgb_model_set_refine(lensgb_model* m, double tau, double kappa) {
    if (!m) return fail(LENSGB_ERR_INVALID, "null model");
    if (!(kappa > 0) || !(tau == tau)) return fail(LENSGB_ERR_INVALID, "kappa must be positive");
    m->refine_tau = (float)tau;
    m->refine_kappa = (float)kappa;
    return LENSGB_OK;
}

int lensgb_model_refined_pixels(const lensgb_model* m, void* stream, long long* n) {
    if (!m || !n) return fail(LENSGB_ERR_INVALID, "null model or output");
    *n = 0;
    if (!m->refine_count) return LENSGB_OK;
    unsigned int v = 0;
    cudaError_t e = cudaMemcpyAsync(&v, m->refine_count, sizeof v, cudaMemcpyDeviceToHost,
                                    (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess)
        return fail(LENSGB_ERR_CUDA, std::string("reading the refine count: ") +
                                         cudaGetErrorString(e));
    *n = v;
    return LENSGB_OK;
}

const char* lensgb_last_error(void) { return g_last_error.c_str(); }

int lensgb_model_create(const lensgb_model_desc* d, lensgb_model** out) {
    if (!d || !out) return fail(LENSGB_ERR_INVALID, "null descriptor or output pointer");
    *out = nullptr;
    if (d->n_lens < 0 || d->n_lens > LENSGB_MAX_PROFILES || d->n_source < 0 ||
        d->n_source > LENSGB_MAX_PROFILES || d->n_lens_light < 0 ||
        d->n_lens_light > LENSGB_MAX_PROFILES)
        return fail(LENSGB_ERR_INVALID, "profile count out of range (0..8 per list)");
    if (d->nx <= 0 || d->ny <= 0 || d->supersampling < 1)
        return fail(LENSGB_ERR_INVALID, "grid size and supersampling must be positive");
    if (d->supersampling > 32)
        return fail(LENSGB_ERR_INVALID, "supersampling factor above 32 is not supported");
    if ((long long)d->nx * d->supersampling > (1 << 22) ||
        (long long)d->ny * d->supersampling > (1 << 22))
        return fail(LENSGB_ERR_INVALID, "supersampled grid side exceeds 2^22");
    if ((long long)d->nx * d->ny * d->supersampling * d->supersampling >= (1LL << 31))
        return fail(LENSGB_ERR_INVALID, "more than 2^31 supersampled rays per system");
    if (d->precision != LENSGB_FP64 && d->precision != LENSGB_FP32_SPLIT)
        return fail(LENSGB_ERR_UNSUPPORTED, "unknown precision mode");
    if (d->psf_type != LENSGB_PSF_NONE && d->psf_type != LENSGB_PSF_PIXEL &&
        d->psf_type != LENSGB_PSF_GAUSSIAN)
        return fail(LENSGB_ERR_UNSUPPORTED, "psf_type must be NONE, PIXEL or GAUSSIAN");
    if (d->psf_type != LENSGB_PSF_NONE && (d->kernel_size < 1 || d->kernel_size % 2 == 0 ||
                                           d->kernel_size > 255))
        return fail(LENSGB_ERR_INVALID, "kernel_size must be odd and in 1..255");
    if (d->low_res_kernel_size != 0 &&
        (d->psf_type != LENSGB_PSF_PIXEL || !d->supersampling_convolution ||
         d->low_res_kernel_size < 1 || d->low_res_kernel_size % 2 == 0 ||
         d->low_res_kernel_size > 255))
        return fail(LENSGB_ERR_INVALID,
                    "low_res_kernel_size must be 0, or odd in 1..255 for PIXEL models with "
                    "supersampling_convolution");
    lensgb_model* m = new lensgb_model();
    m->desc = *d;
    StackDesc& st = m->st;
    st.n_lens = d->n_lens;
    st.n_src = d->n_source;
    st.n_ll = d->n_lens_light;
    int off = 0;
    st.n_epl = 0;
    for (int i = 0; i < MAX_PROF; ++i) {
        st.lens[i] = st.src[i] = st.ll[i] = 0;
        st.lens_off[i] = st.src_off[i] = st.ll_off[i] = 0;
        st.epl_slot[i] = -1;
        st.src_scale[i] = 1.0;
    }
    for (int i = 0; i < d->n_lens; ++i) {
        int c = lens_param_count(d->lens_codes[i]);
        if (c < 0) {
            delete m;
            return fail(LENSGB_ERR_UNSUPPORTED, "unsupported lens profile code");
        }
        st.lens[i] = d->lens_codes[i];
        st.lens_off[i] = off;
        off += c;
        if (d->lens_codes[i] == LENSGB_LENS_EPL ||
            d->lens_codes[i] == LENSGB_LENS_EPL_MULTIPOLE_M1M3M4 ||
            d->lens_codes[i] == LENSGB_LENS_NFW_ELLIPSE_CSE)
            st.epl_slot[i] = st.n_epl++;
    }
    for (int i = 0; i < d->n_source; ++i) {
        int c = light_param_count(d->source_codes[i]);
        if (c < 0) {
            delete m;
            return fail(LENSGB_ERR_UNSUPPORTED, "unsupported source light profile code");
        }
        st.src[i] = d->source_codes[i];
        st.src_off[i] = off;
        st.src_scale[i] = d->deflection_scaling[i];
        off += c;
    }
    for (int i = 0; i < d->n_lens_light; ++i) {
        int c = light_param_count(d->lens_light_codes[i]);
        if (c < 0) {
            delete m;
            return fail(LENSGB_ERR_UNSUPPORTED, "unsupported lens light profile code");
        }
        st.ll[i] = d->lens_light_codes[i];
        st.ll_off[i] = off;
        off += c;
    }
    st.n_params = off;
    st.alpha_scaling = d->alpha_scaling;
    st.flux_scaling = d->flux_scaling;
    st.alpha_scaling_f = (float)d->alpha_scaling;
    st.flux_scaling_f = (float)d->flux_scaling;
    for (int i = 0; i < MAX_PROF; ++i) st.src_scale_f[i] = (float)st.src_scale[i];

    const double* M = d->transform_pix2angle;
    const int s = d->supersampling;
    set_grids(m, d->nx, d->ny, d->ra_at_xy_0, d->dec_at_xy_0);
    m->pixel_width = sqrt(fabs(M[0] * M[3] - M[1] * M[2]));
    m->hr_conv = d->supersampling_convolution != 0 && s > 1 && d->psf_type != LENSGB_PSF_NONE;
    *out = m;
    return LENSGB_OK;
}

int lensgb_model_set_subframe(lensgb_model* m, int row0, int col0, int n,
                              const unsigned char* mask) {
    if (!m) return fail(LENSGB_ERR_INVALID, "null model");
    if (n < 1 || row0 < 0 || col0 < 0 || row0 + n > m->desc.ny || col0 + n > m->desc.nx)
        return fail(LENSGB_ERR_INVALID, "sub-frame outside the image");
    free_scratch(m);
    cudaFree(m->sub_mask);
    m->sub_mask = nullptr;
    if (mask) {
        if (cudaMalloc(&m->sub_mask, (size_t)n * n) != cudaSuccess ||
            cudaMemcpy(m->sub_mask, mask, (size_t)n * n, cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaGetLastError();
            cudaFree(m->sub_mask);
            m->sub_mask = nullptr;
            return fail(LENSGB_ERR_OOM, "sub-frame mask allocation failed");
        }
    }
    // the sub-frame's pixel (0, 0) sits at map_pix2coord(row0, col0): the
    // reference passes the row index in the pixel-x slot (numerics_subframe.py:185-190)
    const double* M = m->desc.transform_pix2angle;
    set_grids(m, n, n, m->desc.ra_at_xy_0 + M[0] * row0 + M[1] * col0,
              m->desc.dec_at_xy_0 + M[2] * row0 + M[3] * col0);
    m->sub = true;
    m->sub_r0 = row0;
    m->sub_c0 = col0;
    return LENSGB_OK;
}

static int ensure_grad_scratch(lensgb_model* m, int n_inst);

int lensgb_model_destroy(lensgb_model* m) {
    if (!m) return LENSGB_OK;
    free_scratch(m);
    free_grad_scratch(m);
    cudaFree(m->sub_mask);
    cudaFree(m->mix_tab);
    cudaFree(m->mix_low);
    cudaFree(m->mix_list);
    if (m->mix_ev) {
        cudaEventSynchronize(m->mix_ev);
        cudaEventDestroy(m->mix_ev);
    }
    cudaFreeHost(m->mix_host);
    if (m->pipe_stream) {
        cudaStreamSynchronize(m->pipe_stream);
        cudaStreamDestroy(m->pipe_stream);
    }
    for (cudaEvent_t e : m->pipe_ev)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : m->pipe_slot_ev)
        if (e) cudaEventDestroy(e);
    if (m->pipe_wait_ev) cudaEventDestroy(m->pipe_wait_ev);
    cudaFree(m->pipe_rows);
    cudaFree(m->pipe_psf);
    cudaFree(m->pipe_out[0]);
    cudaFree(m->pipe_out[1]);
    cudaFree(m->fft_scratch);
    delete m;
    return LENSGB_OK;
}

int lensgb_model_param_count(const lensgb_model* m) { return m ? m->st.n_params : -1; }

int lensgb_model_reserve(lensgb_model* m, int n_inst) {
    if (!m) return fail(LENSGB_ERR_INVALID, "null model");
    if (n_inst < 0 || n_inst > 65535) return fail(LENSGB_ERR_INVALID, "n_inst must be in 0..65535");
    return n_inst > 0 ? ensure_scratch(m, n_inst) : LENSGB_OK;
}

}  // extern "C"

// Images of the model's kernel grid (the sub-frame of sub-frame models) into
// `out`, with the evaluation mask applied before the convolution.
// The tuned ray-kernel pixels per thread for a call of n_inst systems: a
// shape tuned on a large batch is kept off much smaller calls (0: built-in).
static int tuned_ppt(const lensgb_model* m, int n_inst) {
    const long long pix = (long long)n_inst * m->grid.nx * m->grid.ny;
    return (m->tune_ppt > 0 && 4 * pix >= m->tune_pix) ? m->tune_ppt : 0;
}

// Whether a convolution of this model runs by FFT (fftconv.cu) rather than by
// the direct halo-tile kernels (conv.cu).  LENSGB_CONV_AUTO: the FFT only where
// the direct kernels' tile does not fit in shared memory (kernels wider than
// ~140 pixels in FP32, ~100 in FP64), so that every image a model computes
// with the direct kernels -- alone, batched, in mixed-grid launches and served
// -- keeps one summation order.  Measured on GB300 (the bench's convolution
// table), the direct kernels win every FP32 case they can run; FP64 models
// gain from LENSGB_CONV_FFT from K ~ 21 at 180 x 180 (3x at K = 41, 11x at
// K = 85 on 1200 x 1200).
static bool conv_by_fft(const lensgb_model* m, int ny, int nx, int K, int edge) {
    if (m->conv_method == LENSGB_CONV_DIRECT) return false;
    if (fft_conv_size(ny, nx, K, edge) > 4096) return false;
    if (m->conv_method == LENSGB_CONV_FFT) return true;
    return !direct_conv_fits(K, m->desc.precision);
}

// The model's "same"-mode convolution of n_inst (ny, nx) images: FFT or direct.
static int model_conv(lensgb_model* m, const void* in, void* out, const void* psf,
                      long long psf_stride, int n_inst, int ny, int nx, int K, int edge,
                      cudaStream_t s, int tile_rows = 0) {
    if (!conv_by_fft(m, ny, nx, K, edge))
        return launch_conv(in, out, psf, psf_stride, n_inst, ny, nx, K, edge, m->desc.precision,
                           s, tile_rows);
    const size_t need = fft_conv_scratch_bytes(n_inst, ny, nx, K, psf_stride, edge);
    if (need > m->fft_cap) {
        // the previous scratch may still be in use by queued work on this stream
        if (m->fft_scratch) cudaStreamSynchronize(s);
        cudaFree(m->fft_scratch);
        m->fft_scratch = nullptr;
        m->fft_cap = 0;
        if (cudaMalloc(&m->fft_scratch, need) != cudaSuccess) {
            cudaGetLastError();
            return -3;
        }
        m->fft_cap = need;
    }
    return launch_conv_fft(in, out, psf, psf_stride, n_inst, ny, nx, K, edge, m->desc.precision,
                           m->fft_scratch, s);
}

static int conv_fail(int rc) {
    return rc == -3 ? fail(LENSGB_ERR_OOM, "device allocation of FFT convolution scratch failed")
                    : fail(LENSGB_ERR_CUDA, "convolution shared-memory configuration failed");
}

static int image_core(lensgb_model* m, const double* params, int n_inst, const void* psf,
                      long long psf_stride, void* out, int flags, cudaStream_t s) {
    const bool conv = !(flags & LENSGB_UNCONVOLVED) && m->desc.psf_type != LENSGB_PSF_NONE;
    int rc;
    launch_prepare(m->grid, m->st, params, n_inst, m->rec_d, m->rec_f, m->coef_d, m->coef_f, s);
    if ((rc = check_cuda("prepare launch"))) return rc;
    if (conv && m->hr_conv) {
        // supersampled image (one ray per element), convolution on the
        // supersampled grid, then the s x s block mean times the pixel area
        // (SubgridKernelConvolution.re_size_convolve, convolution.py:154-166;
        // GaussianConvolution.re_size_convolve, :237-250)
        RefineArgs rf = refine_args(m, n_inst, m->refine_list, m->refine_count);
        if (rf.tau > 0.f &&
            cudaMemsetAsync(m->refine_count, 0, sizeof(unsigned int), s) != cudaSuccess)
            return check_cuda("refine counter reset");
        launch_raytrace(m->grid_hr, m->st, n_inst, m->rec_d, m->rec_f, m->coef_d, m->coef_f,
                        m->hr_img, flags, 1.0, m->desc.precision, rf, s);
        if ((rc = check_cuda("raytrace launch"))) return rc;
        if (m->sub_mask)
            launch_mask(m->hr_img, n_inst, m->grid.ny, m->grid.nx, m->grid.s, m->sub_mask,
                        m->desc.precision, s);
        if ((rc = model_conv(m, m->hr_img, m->hr_out, psf, psf_stride, n_inst, m->grid_hr.ny,
                             m->grid_hr.nx, m->desc.kernel_size,
                             m->desc.psf_type == LENSGB_PSF_GAUSSIAN ? 1 : 0, s)))
            return conv_fail(rc);
        if ((rc = check_cuda("convolution launch"))) return rc;
        const double area = m->pixel_width * m->pixel_width;
        const int KL = m->desc.low_res_kernel_size;
        if (KL == 0) {
            launch_resize(m->hr_out, out, n_inst, m->grid.ny, m->grid.nx, m->grid.s, area,
                          m->desc.precision, s);
            return check_cuda("re-binning launch");
        }
        // split kernel: re_size(conv_high(hr)) + conv_low(re_size(hr)), then x area
        const size_t esz = m->desc.precision == LENSGB_FP64 ? 8 : 4;
        const void* klow = (const unsigned char*)psf +
                           (size_t)m->desc.kernel_size * m->desc.kernel_size * esz;
        launch_resize(m->hr_out, out, n_inst, m->grid.ny, m->grid.nx, m->grid.s, 1.0,
                      m->desc.precision, s);
        launch_resize(m->hr_img, m->lowres, n_inst, m->grid.ny, m->grid.nx, m->grid.s, 1.0,
                      m->desc.precision, s);
        if ((rc = model_conv(m, m->lowres, m->hr_out, klow, psf_stride, n_inst, m->grid.ny,
                             m->grid.nx, KL, 0, s)))
            return conv_fail(rc);
        launch_add_scaled(out, m->hr_out, (long long)n_inst * m->grid.nx * m->grid.ny, area,
                          m->desc.precision, s);
        return check_cuda("re-binning launch");
    }
    const double scale = m->pixel_width * m->pixel_width;
    void* target = conv ? m->lowres : out;
    RefineArgs rf = refine_args(m, n_inst, m->refine_list, m->refine_count);
    if (rf.tau > 0.f && cudaMemsetAsync(m->refine_count, 0, sizeof(unsigned int), s) != cudaSuccess)
        return check_cuda("refine counter reset");
    launch_raytrace(m->grid, m->st, n_inst, m->rec_d, m->rec_f, m->coef_d, m->coef_f, target,
                    flags, scale, m->desc.precision, rf, s, nullptr, 0, tuned_ppt(m, n_inst));
    if ((rc = check_cuda("raytrace launch"))) return rc;
    if (m->sub_mask)
        launch_mask(target, n_inst, m->grid.ny, m->grid.nx, 1, m->sub_mask, m->desc.precision, s);
    if (conv) {
        if ((rc = model_conv(m, m->lowres, out, psf, psf_stride, n_inst, m->grid.ny, m->grid.nx,
                             m->desc.kernel_size,
                             m->desc.psf_type == LENSGB_PSF_GAUSSIAN ? 1 : 0, s, m->tune_rows)))
            return conv_fail(rc);
        if ((rc = check_cuda("convolution launch"))) return rc;
    }
    return LENSGB_OK;
}

namespace lensgb {

MixedLayout mixed_layout(int cap) {
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    const size_t n = (size_t)(cap > 0 ? cap : 1);
    MixedLayout L;
    L.cap = (int)n;
    L.o_n = 0;
    L.o_grid = 256;
    L.o_off = al(L.o_grid + n * sizeof(GridDesc));
    L.o_koff = al(L.o_off + (n + 1) * 8);
    L.o_ks = al(L.o_koff + n * 8);
    L.o_scale = al(L.o_ks + n * 4);
    L.o_rsys = al(L.o_scale + n * 8);
    L.o_rtoff = al(L.o_rsys + MIX_RAY_GROUPS * n * 4);
    L.o_rcnt = al(L.o_rtoff + MIX_RAY_GROUPS * (n + 1) * 4);
    L.o_gsys = al(L.o_rcnt + MIX_RAY_GROUPS * 4);
    L.o_goff = al(L.o_gsys + MIX_CONV_GROUPS * n * 4);
    L.o_gcnt = al(L.o_goff + MIX_CONV_GROUPS * (n + 1) * 4);
    L.bytes = al(L.o_gcnt + MIX_CONV_GROUPS * 4);
    return L;
}

// Ray group of a supersampling factor (see MIX_RAY_GROUPS).
static int ray_group(int s, bool fp64) { return (!fp64 && s >= 1 && s <= 4) ? s : 0; }

// Convolution group of a kernel width: FP64 has one (run-time width); FP32
// groups 1..6 run the kernel specialised for widths <= 8 g, 7 the run-time-width one.
static int conv_group(int K, bool fp64) {
    if (fp64) return 0;
    const int g = (K + 7) / 8;
    return g > 6 ? 7 : g;
}

int mixed_fill(const lensgb_model* m, unsigned char* H, const MixedLayout& L,
               const lensgb_system_grid* grids, int n, bool conv, MixedCounts* out) {
    if (n < 1 || n > L.cap) return fail(LENSGB_ERR_INVALID, "mixed table capacity exceeded");
    const int s_model = m->desc.supersampling;
    const bool fp64 = m->desc.precision == LENSGB_FP64;
    const int TW = fp64 ? 32 : 64, TH = 64;  // convolution tile (columns, rows)
    GridDesc* gd = (GridDesc*)(H + L.o_grid);
    long long* off = (long long*)(H + L.o_off);
    long long* koff = (long long*)(H + L.o_koff);
    int* ks = (int*)(H + L.o_ks);
    double* area = (double*)(H + L.o_scale);
    int* rsys = (int*)(H + L.o_rsys);
    int* rtoff = (int*)(H + L.o_rtoff);
    int* rcnt = (int*)(H + L.o_rcnt);
    int* gsys = (int*)(H + L.o_gsys);
    int* goff = (int*)(H + L.o_goff);
    int* gcnt = (int*)(H + L.o_gcnt);
    MixedCounts c;
    memset(&c, 0, sizeof c);
    for (int k = 0; k < MIX_RAY_GROUPS; ++k) {
        rcnt[k] = 0;
        rtoff[(size_t)k * (L.cap + 1)] = 0;
    }
    for (int k = 0; k < MIX_CONV_GROUPS; ++k) {
        gcnt[k] = 0;
        goff[(size_t)k * (L.cap + 1)] = 0;
    }
    long long pix = 0, kel = 0, tiles = 0;
    for (int i = 0; i < n; ++i) {
        const lensgb_system_grid& q = grids[i];
        const int s = q.supersampling > 0 ? q.supersampling : s_model;
        if (q.supersampling < 0 || s > 32)
            return fail(LENSGB_ERR_INVALID, "system " + std::to_string(i) +
                                                ": supersampling must be in 0..32");
        if (q.nx <= 0 || q.ny <= 0 || (long long)q.nx * s > (1 << 22) ||
            (long long)q.ny * s > (1 << 22) || (long long)q.nx * q.ny * s * s >= (1LL << 31))
            return fail(LENSGB_ERR_INVALID, "system " + std::to_string(i) + ": bad grid size");
        if (conv && (q.kernel_size < 1 || q.kernel_size % 2 == 0 || q.kernel_size > 255))
            return fail(LENSGB_ERR_INVALID, "system " + std::to_string(i) + ": bad kernel size");
        gd[i] = make_grid(q.nx, q.ny, s, q.transform_pix2angle, q.ra_at_xy_0, q.dec_at_xy_0);
        const double* Mq = q.transform_pix2angle;
        const double pw = sqrt(fabs(Mq[0] * Mq[3] - Mq[1] * Mq[2]));
        area[i] = pw * pw;  // as the single-grid path forms pixel_width^2
        const long long np = (long long)q.nx * q.ny;
        off[i] = pix;
        koff[i] = kel;
        ks[i] = conv ? q.kernel_size : 0;
        pix += np;
        const long long rt = (np + 255) / 256;
        tiles += rt;
        const int rg = ray_group(s, fp64);
        int* ro = rtoff + (size_t)rg * (L.cap + 1);
        rsys[(size_t)rg * L.cap + rcnt[rg]] = i;
        ro[rcnt[rg] + 1] = ro[rcnt[rg]] + (int)rt;
        rcnt[rg]++;
        c.ray_tiles[rg] += (int)rt;
        if (conv) {
            kel += (long long)q.kernel_size * q.kernel_size;
            const int g = conv_group(q.kernel_size, fp64);
            const long long ct = (long long)((q.ny + TH - 1) / TH) * ((q.nx + TW - 1) / TW);
            int* go = goff + (size_t)g * (L.cap + 1);
            gsys[(size_t)g * L.cap + gcnt[g]] = i;
            go[gcnt[g] + 1] = go[gcnt[g]] + (int)ct;
            gcnt[g]++;
            c.conv_tiles[g] += (int)ct;
            c.kmax[g] = std::max(c.kmax[g], q.kernel_size);
        }
    }
    if (pix >= (1LL << 32)) return fail(LENSGB_ERR_INVALID, "more than 2^32 pixels in one call");
    if (tiles >= (1LL << 31)) return fail(LENSGB_ERR_INVALID, "too many ray tiles in one call");
    off[n] = pix;
    *(int*)(H + L.o_n) = n;
    c.n = n;
    c.pix = pix;
    c.kel = kel;
    *out = c;
    return LENSGB_OK;
}

int mixed_reserve(lensgb_model* m, int cap, long long pix, size_t table_bytes) {
    int rc = ensure_scratch(m, cap);
    if (rc) return rc;
    const size_t esz = m->desc.precision == LENSGB_FP64 ? 8 : 4;
    if (table_bytes > m->mix_tab_cap || (size_t)pix > m->mix_pix_cap) {
        cudaFree(m->mix_tab);
        cudaFree(m->mix_low);
        cudaFree(m->mix_list);
        m->mix_tab = nullptr;
        m->mix_low = nullptr;
        m->mix_list = nullptr;
        const size_t tc = std::max(table_bytes, m->mix_tab_cap);
        const size_t pc = std::max((size_t)pix, m->mix_pix_cap);
        m->mix_tab_cap = m->mix_pix_cap = 0;
        if (cudaMalloc(&m->mix_tab, tc) != cudaSuccess ||
            cudaMalloc(&m->mix_low, pc * esz) != cudaSuccess ||
            cudaMalloc(&m->mix_list, pc * sizeof(unsigned int)) != cudaSuccess) {
            cudaGetLastError();
            return fail(LENSGB_ERR_OOM, "device allocation of mixed-launch scratch failed");
        }
        m->mix_tab_cap = tc;
        m->mix_pix_cap = pc;
    }
    return LENSGB_OK;
}

int mixed_launch(lensgb_model* m, const double* params, int n_cap, const unsigned char* tab,
                 const MixedLayout& L, const MixedGrid& gr, const void* psf, void* out, int flags,
                 cudaStream_t st) {
    const bool conv = !(flags & LENSGB_UNCONVOLVED) && m->desc.psf_type != LENSGB_PSF_NONE;
    const int* n_dev = (const int*)(tab + L.o_n);
    const GridDesc* dgrid = (const GridDesc*)(tab + L.o_grid);
    MixedTab mt;
    mt.grid = dgrid;
    mt.off = (const long long*)(tab + L.o_off);
    mt.scale = (const double*)(tab + L.o_scale);
    mt.n_inst = n_dev;
    launch_prepare(m->grid, m->st, params, n_cap, m->rec_d, m->rec_f, m->coef_d, m->coef_f, st,
                   dgrid, n_dev);
    int rc;
    if ((rc = check_cuda("prepare launch"))) return rc;
    RefineArgs rf = refine_args(m, n_cap, m->mix_list, m->refine_count);
    if (rf.tau > 0.f && cudaMemsetAsync(m->refine_count, 0, sizeof(unsigned int), st) != cudaSuccess)
        return check_cuda("refine counter reset");
    void* target = conv ? m->mix_low : out;
    int last = -1;
    for (int g = 0; g < MIX_RAY_GROUPS; ++g)
        if (gr.ray_ctas[g] > 0) last = g;
    for (int g = 0; g < MIX_RAY_GROUPS; ++g) {
        if (gr.ray_ctas[g] <= 0) continue;
        mt.sys = (const int*)(tab + L.o_rsys) + (size_t)g * L.cap;
        mt.tile_off = (const int*)(tab + L.o_rtoff) + (size_t)g * (L.cap + 1);
        mt.count = (const int*)(tab + L.o_rcnt) + g;
        mt.s_group = g;
        mt.refine = g == last;  // one FP64 refine pass after all groups
        launch_raytrace(m->grid, m->st, n_cap, m->rec_d, m->rec_f, m->coef_d, m->coef_f, target,
                        flags, m->pixel_width * m->pixel_width, m->desc.precision, rf, st, &mt,
                        gr.ray_ctas[g]);
    }
    if ((rc = check_cuda("raytrace launch"))) return rc;
    if (conv) {
        ConvMixed cm;
        cm.grid = dgrid;
        cm.off = mt.off;
        cm.koff = (const long long*)(tab + L.o_koff);
        cm.ksize = (const int*)(tab + L.o_ks);
        for (int g = 0; g < 8; ++g) {
            if (gr.conv_ctas[g] <= 0) continue;
            cm.sys = (const int*)(tab + L.o_gsys) + (size_t)g * L.cap;
            cm.tile_off = (const int*)(tab + L.o_goff) + (size_t)g * (L.cap + 1);
            cm.count = (const int*)(tab + L.o_gcnt) + g;
            if (launch_conv_mixed(m->mix_low, out, psf, cm, gr.conv_ctas[g], gr.conv_kmax[g],
                                  g == 7 ? 0 : g, m->desc.psf_type == LENSGB_PSF_GAUSSIAN,
                                  m->desc.precision, st))
                return fail(LENSGB_ERR_CUDA, "convolution shared-memory configuration failed");
        }
        if ((rc = check_cuda("convolution launch"))) return rc;
    }
    return LENSGB_OK;
}

}  // namespace lensgb

extern "C" {

int lensgb_image(lensgb_model* m, const double* params, int n_inst, const void* psf,
                 long long psf_stride, void* out, int flags, void* stream) {
    if (!m) return fail(LENSGB_ERR_INVALID, "null model");
    if (n_inst < 0 || n_inst > 65535)
        return fail(LENSGB_ERR_INVALID, "n_inst must be in 0..65535");
    if (n_inst == 0) return LENSGB_OK;
    if (!out || (!params && m->st.n_params > 0))
        return fail(LENSGB_ERR_INVALID, "null params or output pointer");
    const bool conv = !(flags & LENSGB_UNCONVOLVED) && m->desc.psf_type != LENSGB_PSF_NONE;
    if (conv && !psf) return fail(LENSGB_ERR_INVALID, "null PSF kernel pointer");
    if (psf_stride < 0) return fail(LENSGB_ERR_INVALID, "negative PSF stride");
    int rc = check_refine_size(m, n_inst);
    if (rc) return rc;
    rc = ensure_scratch(m, n_inst);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (!m->sub) return image_core(m, params, n_inst, psf, psf_stride, out, flags, s);
    // NumericsSubFrame: the sub-frame image, zeros elsewhere (numerics_subframe.py:87-149)
    rc = image_core(m, params, n_inst, psf, psf_stride, m->sub_out, flags, s);
    if (rc) return rc;
    launch_embed(m->sub_out, out, n_inst, m->grid.nx, m->sub_r0, m->sub_c0, m->desc.ny,
                 m->desc.nx, m->desc.precision, s);
    return check_cuda("sub-frame embedding launch");
}

// Grow-only device buffer.
static int grow_buffer(void** p, size_t* cap, size_t need) {
    if (need <= *cap) return LENSGB_OK;
    cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    if (cudaMalloc(p, need) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return fail(LENSGB_ERR_OOM, "device allocation of host-call staging failed");
    }
    *cap = need;
    return LENSGB_OK;
}

int lensgb_image_host(lensgb_model* m, const double* params, int n_inst, const void* psf,
                      long long psf_stride, void* out, int flags, int n_chunks, void* stream) {
    if (!m) return fail(LENSGB_ERR_INVALID, "null model");
    if (n_inst < 0 || n_inst > 65535)
        return fail(LENSGB_ERR_INVALID, "n_inst must be in 0..65535");
    if (n_inst == 0) return LENSGB_OK;
    if (!out || (!params && m->st.n_params > 0))
        return fail(LENSGB_ERR_INVALID, "null params or output pointer");
    const bool conv = !(flags & LENSGB_UNCONVOLVED) && m->desc.psf_type != LENSGB_PSF_NONE;
    if (conv && !psf) return fail(LENSGB_ERR_INVALID, "null PSF kernel pointer");
    if (psf_stride < 0) return fail(LENSGB_ERR_INVALID, "negative PSF stride");
    if (n_chunks < 0 || n_chunks > 16) return fail(LENSGB_ERR_INVALID, "n_chunks must be in 0..16");
    if (n_chunks == 0) n_chunks = 1;
    if (n_chunks > n_inst) n_chunks = n_inst;
    const size_t esz = m->desc.precision == LENSGB_FP64 ? 8 : 4;
    const size_t P = (size_t)m->st.n_params;
    const size_t npix = (size_t)m->desc.nx * m->desc.ny;
    const size_t k_el = conv ? (size_t)(m->desc.kernel_size * m->desc.kernel_size +
                                        m->desc.low_res_kernel_size * m->desc.low_res_kernel_size)
                             : 0;
    const size_t psf_el = !conv ? 0 : (psf_stride > 0 ? (size_t)psf_stride * n_inst : k_el);
    if (!m->pipe_stream &&
        cudaStreamCreateWithFlags(&m->pipe_stream, cudaStreamNonBlocking) != cudaSuccess)
        return check_cuda("copy stream");
    for (cudaEvent_t& e : m->pipe_ev)
        if (!e && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
            return check_cuda("copy event");
    for (cudaEvent_t& e : m->pipe_slot_ev)
        if (!e && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
            return check_cuda("copy event");
    cudaStream_t st = (cudaStream_t)stream;
    const int slot = m->pipe_slot;
    // this slot's images of two calls ago must have left before it is rewritten
    // (growing a buffer frees it: wait for the copies first)
    if (cudaStreamWaitEvent(st, m->pipe_slot_ev[slot], 0) != cudaSuccess)
        return check_cuda("stream order");
    if (npix * n_inst * esz > m->pipe_out_cap[slot] &&
        cudaEventSynchronize(m->pipe_slot_ev[slot]) != cudaSuccess)
        return check_cuda("copy event");
    int rc;
    if ((rc = grow_buffer(&m->pipe_rows, &m->pipe_rows_cap, P * n_inst * 8 + 8)) ||
        (rc = grow_buffer(&m->pipe_psf, &m->pipe_psf_cap, psf_el * esz + 16)) ||
        (rc = grow_buffer(&m->pipe_out[slot], &m->pipe_out_cap[slot], npix * n_inst * esz)))
        return rc;
    m->pipe_slot ^= 1;
    unsigned char* rows_d = (unsigned char*)m->pipe_rows;
    unsigned char* psf_d = (unsigned char*)m->pipe_psf;
    unsigned char* out_d = (unsigned char*)m->pipe_out[slot];
    // a shared PSF goes up once
    if (conv && psf_stride == 0 &&
        cudaMemcpyAsync(psf_d, psf, k_el * esz, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return check_cuda("PSF copy");
    for (int c = 0; c < n_chunks; ++c) {
        const int i0 = (int)((long long)n_inst * c / n_chunks);
        const int i1 = (int)((long long)n_inst * (c + 1) / n_chunks);
        const int nc = i1 - i0;
        if (nc <= 0) continue;
        if (cudaMemcpyAsync(rows_d + (size_t)i0 * P * 8, params + (size_t)i0 * P, (size_t)nc * P * 8,
                            cudaMemcpyHostToDevice, st) != cudaSuccess)
            return check_cuda("parameter copy");
        const unsigned char* kp = psf_d;
        if (conv && psf_stride > 0) {
            const size_t off = (size_t)i0 * psf_stride * esz;
            if (cudaMemcpyAsync(psf_d + off, (const unsigned char*)psf + off,
                                (size_t)nc * psf_stride * esz, cudaMemcpyHostToDevice,
                                st) != cudaSuccess)
                return check_cuda("PSF copy");
            kp = psf_d + off;
        }
        rc = lensgb_image(m, (const double*)(rows_d + (size_t)i0 * P * 8), nc, conv ? kp : nullptr,
                          psf_stride, out_d + (size_t)i0 * npix * esz, flags, stream);
        if (rc) return rc;
        if (cudaEventRecord(m->pipe_ev[c], st) != cudaSuccess ||
            cudaStreamWaitEvent(m->pipe_stream, m->pipe_ev[c], 0) != cudaSuccess ||
            cudaMemcpyAsync((unsigned char*)out + (size_t)i0 * npix * esz,
                            out_d + (size_t)i0 * npix * esz, (size_t)nc * npix * esz,
                            cudaMemcpyDeviceToHost, m->pipe_stream) != cudaSuccess)
            return check_cuda("image copy");
    }
    // the copies stay in flight on the copy stream (lensgb_image_host_wait)
    if (cudaEventRecord(m->pipe_slot_ev[slot], m->pipe_stream) != cudaSuccess)
        return check_cuda("copy event");
    return LENSGB_OK;
}

int lensgb_image_host_wait(lensgb_model* m, void* stream) {
    if (!m) return fail(LENSGB_ERR_INVALID, "null model");
    if (!m->pipe_stream) return LENSGB_OK;
    if (!m->pipe_wait_ev &&
        cudaEventCreateWithFlags(&m->pipe_wait_ev, cudaEventDisableTiming) != cudaSuccess)
        return check_cuda("copy event");
    if (cudaEventRecord(m->pipe_wait_ev, m->pipe_stream) != cudaSuccess ||
        cudaStreamWaitEvent((cudaStream_t)stream, m->pipe_wait_ev, 0) != cudaSuccess)
        return check_cuda("stream order");
    return LENSGB_OK;
}

int lensgb_model_set_tuning(lensgb_model* m, int ppt, int conv_tile_rows) {
    if (!m) return fail(LENSGB_ERR_INVALID, "null model");
    if (!(ppt == 0 || ppt == 1 || ppt == 2 || ppt == 4 || ppt == 8))
        return fail(LENSGB_ERR_INVALID, "ppt must be 0, 1, 2, 4 or 8");
    if (!(conv_tile_rows == 0 ||
          (conv_tile_rows >= 32 && conv_tile_rows <= 64 && conv_tile_rows % 4 == 0)))
        return fail(LENSGB_ERR_INVALID, "conv_tile_rows must be 0 or a multiple of 4 in 32..64");
    m->tune_ppt = ppt;
    m->tune_rows = conv_tile_rows;
    m->tune_pix = 0;
    return LENSGB_OK;
}

}  // extern "C"

// Minimum over three timed launches of `f` (after one untimed) on stream st.
template <typename F>
static int time_min_ms(cudaStream_t st, cudaEvent_t a, cudaEvent_t b, F f, double* ms) {
    int rc = f();
    if (rc) return rc;
    double best = 1e300;
    for (int r = 0; r < 3; ++r) {
        if (cudaEventRecord(a, st) != cudaSuccess) return check_cuda("autotune event");
        if ((rc = f())) return rc;
        if (cudaEventRecord(b, st) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess)
            return check_cuda("autotune event");
        float t = 0.f;
        cudaEventElapsedTime(&t, a, b);
        best = std::min(best, (double)t);
    }
    *ms = best;
    return LENSGB_OK;
}

extern "C" {

int lensgb_model_autotune(lensgb_model* m, const double* params, int n_inst, const void* psf,
                          long long psf_stride, void* out, void* stream,
                          lensgb_tune_result* result) {
    if (!m || !result) return fail(LENSGB_ERR_INVALID, "null model or result");
    if (n_inst <= 0 || n_inst > 65535) return fail(LENSGB_ERR_INVALID, "n_inst must be in 1..65535");
    if (!out || (!params && m->st.n_params > 0))
        return fail(LENSGB_ERR_INVALID, "null params or output pointer");
    if (m->hr_conv || m->sub)
        return fail(LENSGB_ERR_UNSUPPORTED,
                    "autotune does not take supersampled-convolution or sub-frame models");
    const bool conv = m->desc.psf_type != LENSGB_PSF_NONE;
    if (conv && !psf) return fail(LENSGB_ERR_INVALID, "null PSF kernel pointer");
    if (psf_stride < 0) return fail(LENSGB_ERR_INVALID, "negative PSF stride");
    int rc = check_refine_size(m, n_inst);
    if (rc) return rc;
    if ((rc = ensure_scratch(m, n_inst))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t a = nullptr, b = nullptr;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
        if (a) cudaEventDestroy(a);
        return check_cuda("autotune event");
    }
    memset(result, 0, sizeof *result);
    // ray stage: prepare + rays + refine into `out` (unconvolved)
    const int ppts[5] = {0, 1, 2, 4, 8};
    m->tune_pix = 0;
    double best_ray = 1e300;
    int best_ppt = 0;
    for (int k = 0; k < 5 && rc == LENSGB_OK; ++k) {
        m->tune_ppt = ppts[k];
        double t = 0;
        rc = time_min_ms(st, a, b, [&] {
            return image_core(m, params, n_inst, psf, psf_stride, out, LENSGB_UNCONVOLVED, st);
        }, &t);
        if (rc) break;
        if (k == 0) result->ray_ms_builtin = t;
        if (t < best_ray) {
            best_ray = t;
            best_ppt = ppts[k];
        }
    }
    m->tune_ppt = rc == LENSGB_OK ? best_ppt : 0;
    m->tune_pix = (long long)n_inst * m->grid.nx * m->grid.ny;
    result->ppt = best_ppt;
    result->ray_ms = best_ray;
    if (rc == LENSGB_OK && conv) {
        // convolution stage on the un-convolved images of one full call
        rc = image_core(m, params, n_inst, psf, psf_stride, out, 0, st);
        const bool fp32 = m->desc.precision == LENSGB_FP32_SPLIT;
        double best_conv = 1e300;
        int best_rows = 0;
        for (int rows = 0; rc == LENSGB_OK && rows <= (fp32 ? 64 : 0); rows += (rows ? 4 : 32)) {
            double t = 0;
            rc = time_min_ms(st, a, b, [&] {
                if (launch_conv(m->lowres, out, psf, psf_stride, n_inst, m->grid.ny, m->grid.nx,
                                m->desc.kernel_size,
                                m->desc.psf_type == LENSGB_PSF_GAUSSIAN ? 1 : 0,
                                m->desc.precision, st, rows))
                    return fail(LENSGB_ERR_CUDA, "convolution shared-memory configuration failed");
                return check_cuda("convolution launch");
            }, &t);
            if (rc) break;
            if (rows == 0) result->conv_ms_builtin = t;
            if (t < best_conv) {
                best_conv = t;
                best_rows = rows;
            }
        }
        m->tune_rows = rc == LENSGB_OK ? best_rows : 0;
        result->conv_tile_rows = best_rows;
        result->conv_ms = best_conv;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return rc;
}

int lensgb_image_mixed(lensgb_model* m, const double* params, int n_inst,
                       const lensgb_system_grid* grids, const void* psf, void* out, int flags,
                       void* stream) {
    if (!m) return fail(LENSGB_ERR_INVALID, "null model");
    if (n_inst < 0 || n_inst > 65535)
        return fail(LENSGB_ERR_INVALID, "n_inst must be in 0..65535");
    if (n_inst == 0) return LENSGB_OK;
    if (!out || !grids || (!params && m->st.n_params > 0))
        return fail(LENSGB_ERR_INVALID, "null params, grids or output pointer");
    if (m->hr_conv || m->sub)
        return fail(LENSGB_ERR_UNSUPPORTED,
                    "lensgb_image_mixed does not take supersampled-convolution or sub-frame models");
    const bool conv = !(flags & LENSGB_UNCONVOLVED) && m->desc.psf_type != LENSGB_PSF_NONE;
    if (conv && !psf) return fail(LENSGB_ERR_INVALID, "null PSF kernel pointer");
    const MixedLayout L = mixed_layout(n_inst);
    // the host tables: wait for the previous table copy to have read them
    if (m->mix_ev_pending && cudaEventSynchronize(m->mix_ev) != cudaSuccess)
        return check_cuda("mixed table event");
    m->mix_ev_pending = false;
    if (!m->mix_ev && cudaEventCreateWithFlags(&m->mix_ev, cudaEventDisableTiming) != cudaSuccess)
        return check_cuda("mixed table event");
    if (L.bytes > m->mix_host_cap) {
        cudaFreeHost(m->mix_host);
        m->mix_host = nullptr;
        m->mix_host_cap = 0;
        if (cudaMallocHost(&m->mix_host, L.bytes) != cudaSuccess) {
            cudaGetLastError();
            return fail(LENSGB_ERR_OOM, "page-locked allocation of mixed-launch tables failed");
        }
        m->mix_host_cap = L.bytes;
    }
    MixedCounts c;
    int rc = mixed_fill(m, m->mix_host, L, grids, n_inst, conv, &c);
    if (rc) return rc;
    if ((rc = mixed_reserve(m, n_inst, c.pix, L.bytes))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemcpyAsync(m->mix_tab, m->mix_host, L.bytes, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaEventRecord(m->mix_ev, st) != cudaSuccess)
        return check_cuda("mixed table copy");
    m->mix_ev_pending = true;
    // one CTA per tile; every group with tiles gets its launch
    MixedGrid gr;
    for (int k = 0; k < MIX_RAY_GROUPS; ++k) gr.ray_ctas[k] = c.ray_tiles[k];
    for (int k = 0; k < 8; ++k) {
        gr.conv_ctas[k] = c.conv_tiles[k];
        gr.conv_kmax[k] = c.kmax[k];
    }
    return mixed_launch(m, params, n_inst, m->mix_tab, L, gr, psf, out, flags, st);
}

int lensgb_convolve(const lensgb_model* m, const void* in, int n_inst, const void* psf,
                    long long psf_stride, void* out, void* stream) {
    if (!m) return fail(LENSGB_ERR_INVALID, "null model");
    if (n_inst < 0 || n_inst > 65535)
        return fail(LENSGB_ERR_INVALID, "n_inst must be in 0..65535");
    if (m->desc.psf_type == LENSGB_PSF_NONE)
        return fail(LENSGB_ERR_INVALID, "model has psf_type NONE");
    if (n_inst == 0) return LENSGB_OK;
    if (!in || !out || !psf) return fail(LENSGB_ERR_INVALID, "null image or PSF pointer");
    if (in == out) return fail(LENSGB_ERR_INVALID, "in-place convolution is not supported");
    if (psf_stride < 0) return fail(LENSGB_ERR_INVALID, "negative PSF stride");
    const int rc = model_conv(const_cast<lensgb_model*>(m), in, out, psf, psf_stride, n_inst,
                              m->desc.ny, m->desc.nx, m->desc.kernel_size,
                              m->desc.psf_type == LENSGB_PSF_GAUSSIAN ? 1 : 0,
                              (cudaStream_t)stream, m->tune_rows);
    if (rc) return conv_fail(rc);
    return check_cuda("convolution launch");
}

int lensgb_model_set_convolution(lensgb_model* m, int method) {
    if (!m) return fail(LENSGB_ERR_INVALID, "null model");
    if (method != LENSGB_CONV_AUTO && method != LENSGB_CONV_DIRECT && method != LENSGB_CONV_FFT)
        return fail(LENSGB_ERR_INVALID, "method must be LENSGB_CONV_AUTO, _DIRECT or _FFT");
    m->conv_method = method;
    return LENSGB_OK;
}

int lensgb_model_set_grad_precision(lensgb_model* m, int precision) {
    if (!m) return fail(LENSGB_ERR_INVALID, "null model");
    if (precision != LENSGB_FP64 && precision != LENSGB_FP32_SPLIT)
        return fail(LENSGB_ERR_INVALID, "precision must be LENSGB_FP64 or LENSGB_FP32_SPLIT");
    m->grad_precision = precision;
    return LENSGB_OK;
}

int lensgb_set_conv_tma(int enable) {
    set_conv_tma(enable);
    return LENSGB_OK;
}

int lensgb_wait_timeouts(unsigned int* count) {
    if (!count) return fail(LENSGB_ERR_INVALID, "null count pointer");
    *count = conv_wait_timeouts();
    return check_cuda("wait-timeout counter read");
}

int lensgb_loglike(lensgb_model* m, const double* params, int n_inst, const void* psf,
                   long long psf_stride, const lensgb_noise_desc* nd, void* image_out,
                   double* logl, void* stream) {
    if (!m) return fail(LENSGB_ERR_INVALID, "null model");
    if (!nd || !nd->data_dev) return fail(LENSGB_ERR_INVALID, "null noise description or data");
    if (!image_out || !logl) return fail(LENSGB_ERR_INVALID, "null image or logL output");
    if (!nd->noise_map_dev && !nd->exposure_map_dev && !(nd->exposure_time > 0))
        return fail(LENSGB_ERR_INVALID, "exposure time must be positive without a noise map");
    if (nd->data_stride < 0 || nd->noise_stride < 0 || nd->exposure_stride < 0 ||
        nd->mask_stride < 0)
        return fail(LENSGB_ERR_INVALID, "negative stride");
    int rc = lensgb_image(m, params, n_inst, psf, psf_stride, image_out, 0, stream);
    if (rc) return rc;
    if (n_inst == 0) return LENSGB_OK;
    LoglikeArgs a;
    a.data = nd->data_dev;
    a.data_stride = nd->data_stride;
    a.mask = nd->mask_dev;
    a.mask_stride = nd->mask_stride;
    a.noise_map = nd->noise_map_dev;
    a.noise_stride = nd->noise_stride;
    a.exposure = nd->exposure_map_dev;
    a.exposure_stride = nd->exposure_stride;
    a.exposure_time = nd->exposure_time;
    a.background_rms = nd->background_rms;
    a.error_map = nd->error_map_dev;
    launch_loglike(image_out, n_inst, (long long)m->desc.nx * m->desc.ny, a, logl,
                   m->desc.precision, (cudaStream_t)stream);
    return check_cuda("likelihood launch");
}

int lensgb_loglike_image(const lensgb_model* m, const void* image, int n_inst,
                         const lensgb_noise_desc* nd, double* logl, void* stream) {
    if (!m) return fail(LENSGB_ERR_INVALID, "null model");
    if (n_inst < 0) return fail(LENSGB_ERR_INVALID, "negative system count");
    if (n_inst == 0) return LENSGB_OK;
    if (!nd || !nd->data_dev) return fail(LENSGB_ERR_INVALID, "null noise description or data");
    if (!image || !logl) return fail(LENSGB_ERR_INVALID, "null image or logL pointer");
    if (!nd->noise_map_dev && !nd->exposure_map_dev && !(nd->exposure_time > 0))
        return fail(LENSGB_ERR_INVALID, "exposure time must be positive without a noise map");
    if (nd->data_stride < 0 || nd->noise_stride < 0 || nd->exposure_stride < 0 ||
        nd->mask_stride < 0)
        return fail(LENSGB_ERR_INVALID, "negative stride");
    LoglikeArgs a;
    a.data = nd->data_dev;
    a.data_stride = nd->data_stride;
    a.mask = nd->mask_dev;
    a.mask_stride = nd->mask_stride;
    a.noise_map = nd->noise_map_dev;
    a.noise_stride = nd->noise_stride;
    a.exposure = nd->exposure_map_dev;
    a.exposure_stride = nd->exposure_stride;
    a.exposure_time = nd->exposure_time;
    a.background_rms = nd->background_rms;
    a.error_map = nd->error_map_dev;
    launch_loglike(image, n_inst, (long long)m->desc.nx * m->desc.ny, a, logl, m->desc.precision,
                   (cudaStream_t)stream);
    return check_cuda("likelihood launch");
}

int lensgb_point_sources_add(const lensgb_model* m, const double* ps, int n_images, int n_inst,
                             const double* kernel, int kernel_size, long long kernel_stride,
                             int subgrid, void* image, void* stream) {
    if (!m) return fail(LENSGB_ERR_INVALID, "null model");
    if (n_images < 0 || n_inst < 0 || n_inst > 65535)
        return fail(LENSGB_ERR_INVALID, "n_images >= 0 and n_inst in 0..65535 required");
    if (n_images == 0 || n_inst == 0) return LENSGB_OK;
    if (!ps || !kernel || !image) return fail(LENSGB_ERR_INVALID, "null point, kernel or image");
    if (kernel_size < 1 || kernel_size % 2 == 0)
        return fail(LENSGB_ERR_INVALID, "kernel dimensions must be odd");
    if (kernel_stride != 0 && kernel_stride < (long long)kernel_size * kernel_size)
        return fail(LENSGB_ERR_INVALID, "kernel stride smaller than one kernel");
    if (subgrid < 1) return fail(LENSGB_ERR_INVALID, "subgrid factor must be >= 1");
    if (m->sub)
        return fail(LENSGB_ERR_UNSUPPORTED, "point sources on a sub-frame model");
    // PixelGrid: Ma2pix = inverse(transform_pix2angle), pixel position of ra = dec = 0
    const double* T = m->desc.transform_pix2angle;
    const double det = T[0] * T[3] - T[1] * T[2];
    if (!(det != 0.0)) return fail(LENSGB_ERR_INVALID, "singular pixel transform");
    const double M[4] = {T[3] / det, -T[1] / det, -T[2] / det, T[0] / det};
    const double ra0 = -m->desc.ra_at_xy_0, dec0 = -m->desc.dec_at_xy_0;
    const double x0 = M[0] * ra0 + M[1] * dec0, y0 = M[2] * ra0 + M[3] * dec0;
    launch_point_sources(ps, n_images, n_inst, kernel, kernel_size, kernel_stride, subgrid, M, x0,
                         y0, m->desc.ny, m->desc.nx, m->desc.flux_scaling, image,
                         m->desc.precision, (cudaStream_t)stream);
    return check_cuda("point-source rendering launch");
}

int lensgb_linear_solve(const lensgb_model* m, const void* A, int n_linear, int n_inst,
                        const lensgb_noise_desc* nd, int flags, double* param, double* cov,
                        void* image_out, double* logl, void* stream) {
    if (!m) return fail(LENSGB_ERR_INVALID, "null model");
    if (n_inst < 0 || n_inst > 65535) return fail(LENSGB_ERR_INVALID, "n_inst must be in 0..65535");
    if (n_linear < 1 || n_linear > LENSGB_LINEAR_MAX)
        return fail(LENSGB_ERR_INVALID, "n_linear must be in 1..8");
    if (flags & ~(LENSGB_LINEAR_INVERSE | LENSGB_LINEAR_POSITIVE))
        return fail(LENSGB_ERR_INVALID, "unknown linear-solve flags");
    if (n_inst == 0) return LENSGB_OK;
    if (!A || !param || !image_out || !logl)
        return fail(LENSGB_ERR_INVALID, "null response, parameter, image or logL pointer");
    if (!nd || !nd->data_dev) return fail(LENSGB_ERR_INVALID, "null noise description or data");
    if (!nd->noise_map_dev && !nd->exposure_map_dev && !(nd->exposure_time > 0))
        return fail(LENSGB_ERR_INVALID, "exposure time must be positive without a noise map");
    if (nd->data_stride < 0 || nd->noise_stride < 0 || nd->exposure_stride < 0 ||
        nd->mask_stride < 0)
        return fail(LENSGB_ERR_INVALID, "negative stride");
    LoglikeArgs a;
    a.data = nd->data_dev;
    a.data_stride = nd->data_stride;
    a.mask = nd->mask_dev;
    a.mask_stride = nd->mask_stride;
    a.noise_map = nd->noise_map_dev;
    a.noise_stride = nd->noise_stride;
    a.exposure = nd->exposure_map_dev;
    a.exposure_stride = nd->exposure_stride;
    a.exposure_time = nd->exposure_time;
    a.background_rms = nd->background_rms;
    a.error_map = nd->error_map_dev;
    launch_linear_solve(A, n_linear, n_inst, (long long)m->desc.nx * m->desc.ny, a, flags, param,
                        (flags & LENSGB_LINEAR_INVERSE) ? cov : nullptr, image_out, logl,
                        m->desc.precision, (cudaStream_t)stream);
    return check_cuda("linear solve launch");
}

static int ensure_grad_scratch(lensgb_model* m, int n_inst) {
    if (n_inst <= m->grad_cap) return LENSGB_OK;
    int cap = m->grad_cap > 0 ? m->grad_cap : 1;
    while (cap < n_inst) cap *= 2;
    free_grad_scratch(m);
    const size_t full = (size_t)m->desc.nx * m->desc.ny;
    const size_t kgrid = (size_t)m->grid.nx * m->grid.ny;
    const bool hr = m->hr_conv;
    const size_t hgrid = hr ? (size_t)m->grid_hr.nx * m->grid_hr.ny : 0;
    const int K = m->desc.kernel_size, KL = m->desc.low_res_kernel_size;
    const size_t kk = (size_t)K * K + (size_t)KL * KL;
    const size_t ncoef = (size_t)cap * (m->st.n_epl > 0 ? m->st.n_epl : 1) * EPL_NMAX;
    const GridDesc& rg = hr ? m->grid_hr : m->grid;
    // two sets of partials: the FP32 pass and the FP64 pass over flagged pixels
    const size_t npart =
        2 * (size_t)cap * grad_chunks(rg) * (m->st.n_params > 0 ? m->st.n_params : 1);
    // one flag byte per ray-grid pixel of each system, allocated as doubles
    const size_t nflag = ((size_t)cap * rg.nx * rg.ny + 7) / 8;
    size_t pad = 0;
    if (m->desc.psf_type == LENSGB_PSF_GAUSSIAN) {
        const size_t side = (size_t)(hr ? m->grid_hr.nx : m->grid.nx) + K - 1;
        const size_t sidey = (size_t)(hr ? m->grid_hr.ny : m->grid.ny) + K - 1;
        pad = side * sidey;
    }
    struct {
        double** p;
        size_t n;
    } want[] = {{&m->g_dcoef, ncoef},         {&m->g_psf, (size_t)cap * (kk > 0 ? kk : 1)},
                {&m->g_m, (size_t)cap * full}, {&m->g_a, (size_t)cap * kgrid},
                {&m->g_b, (size_t)cap * kgrid}, {&m->g_c, (size_t)cap * hgrid},
                {&m->g_d, (size_t)cap * hgrid}, {&m->g_pad_a, (size_t)cap * pad},
                {&m->g_pad_b, (size_t)cap * pad}, {&m->g_partial, npart},
                {&m->g_flag, nflag}};
    for (auto& w : want) {
        if (w.n == 0) continue;
        if (cudaMalloc(w.p, w.n * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            free_grad_scratch(m);
            return fail(LENSGB_ERR_OOM, "device allocation of gradient scratch failed");
        }
    }
    m->grad_cap = cap;
    return LENSGB_OK;
}

int lensgb_loglike_grad(lensgb_model* m, const double* params, int n_inst, const void* psf,
                        long long psf_stride, const lensgb_noise_desc* nd, void* image_out,
                        double* logl, double* grad, void* stream) {
    if (!m) return fail(LENSGB_ERR_INVALID, "null model");
    if (m->desc.precision != LENSGB_FP64)
        return fail(LENSGB_ERR_UNSUPPORTED, "the likelihood gradient needs an FP64 model");
    if (!grad_supported(m->st))
        return fail(LENSGB_ERR_UNSUPPORTED,
                    "the likelihood gradient supports lens stacks of EPL, EPL_MULTIPOLE_M1M3M4, "
                    "SIE, NIE, NFW, TNFW, NFW_ELLIPSE_CSE, CONVERGENCE and SHEAR and Sersic "
                    "light profiles, with at most 64 parameters per system");
    if (!nd || !nd->data_dev) return fail(LENSGB_ERR_INVALID, "null noise description or data");
    if (!image_out || !logl || !grad) return fail(LENSGB_ERR_INVALID, "null output pointer");
    if (!nd->noise_map_dev && !nd->exposure_map_dev && !(nd->exposure_time > 0))
        return fail(LENSGB_ERR_INVALID, "exposure time must be positive without a noise map");
    if (nd->data_stride < 0 || nd->noise_stride < 0 || nd->exposure_stride < 0 ||
        nd->mask_stride < 0)
        return fail(LENSGB_ERR_INVALID, "negative stride");
    int rc = lensgb_image(m, params, n_inst, psf, psf_stride, image_out, 0, stream);
    if (rc) return rc;
    if (n_inst == 0) return LENSGB_OK;
    if ((rc = ensure_grad_scratch(m, n_inst))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    LoglikeArgs a;
    a.data = nd->data_dev;
    a.data_stride = nd->data_stride;
    a.mask = nd->mask_dev;
    a.mask_stride = nd->mask_stride;
    a.noise_map = nd->noise_map_dev;
    a.noise_stride = nd->noise_stride;
    a.exposure = nd->exposure_map_dev;
    a.exposure_stride = nd->exposure_stride;
    a.exposure_time = nd->exposure_time;
    a.background_rms = nd->background_rms;
    a.error_map = nd->error_map_dev;
    // reverse of the forward path: logL and d logL / d image (full frame), the
    // sub-frame crop, the transposed convolution(s) and re-binning, the
    // evaluation mask, then the rays
    const long long full = (long long)m->desc.nx * m->desc.ny;
    launch_grad_weights((const double*)image_out, n_inst, full, a, m->g_m, logl, s);
    const int n = m->grid.nx, ny = m->grid.ny, nx = m->grid.nx;
    double* gk = m->g_m;  // d logL / d (image on the kernel grid)
    if (m->sub) {
        launch_crop(m->g_m, m->g_a, n_inst, n, m->sub_r0, m->sub_c0, m->desc.ny, m->desc.nx, s);
        gk = m->g_a;
    }
    const bool conv = m->desc.psf_type != LENSGB_PSF_NONE;
    const int edge = m->desc.psf_type == LENSGB_PSF_GAUSSIAN ? 1 : 0;
    const int K = m->desc.kernel_size, KL = m->desc.low_res_kernel_size;
    const double area = m->pixel_width * m->pixel_width;
    const double* psf_d = (const double*)psf;
    const char* conv_err = "transposed convolution shared-memory configuration failed";
    if (conv && m->hr_conv) {
        const int S = m->grid.s;
        const int hy = m->grid_hr.ny, hx = m->grid_hr.nx;
        // d out / d hr_out: area / s^2 per supersampled element (re_size), then
        // the supersampled kernel's transpose
        launch_expand(gk, m->g_c, n_inst, ny, nx, S, area / ((double)S * S), 0, s);
        if (launch_conv_transpose(m->g_c, m->g_d, psf_d, psf_stride, K, edge, n_inst, hy, hx,
                                  m->g_psf, m->g_pad_a, m->g_pad_b, s))
            return fail(LENSGB_ERR_CUDA, conv_err);
        if (KL > 0) {
            // split kernel: + re_size^T(conv_low^T(g area)), pixel-scale part
            launch_scale(gk, (long long)n_inst * ny * nx, area, s);
            if (launch_conv_transpose(gk, m->g_b, psf_d + (long long)K * K, psf_stride, KL, 0,
                                      n_inst, ny, nx, m->g_psf + (long long)n_inst * K * K,
                                      nullptr, nullptr, s))
                return fail(LENSGB_ERR_CUDA, conv_err);
            launch_expand(m->g_b, m->g_d, n_inst, ny, nx, S, 1.0 / ((double)S * S), 1, s);
        }
        if (m->sub_mask) launch_mask(m->g_d, n_inst, ny, nx, S, m->sub_mask, LENSGB_FP64, s);
        if (launch_grad_rays(m->grid_hr, m->st, n_inst, params, m->rec_d, m->coef_d, m->g_dcoef,
                             m->g_d, 1.0, m->g_partial, grad, m->grad_precision,
                             (unsigned char*)m->g_flag, m->grad_tau, s))
            return fail(LENSGB_ERR_CUDA, "gradient launch failed");
        return check_cuda("likelihood gradient launch");
    }
    const double* gl = gk;
    if (conv) {
        if (launch_conv_transpose(gk, m->g_b, psf_d, psf_stride, K, edge, n_inst, ny, nx,
                                  m->g_psf, m->g_pad_a, m->g_pad_b, s))
            return fail(LENSGB_ERR_CUDA, conv_err);
        gl = m->g_b;
    }
    if (m->sub_mask) launch_mask((void*)gl, n_inst, ny, nx, 1, m->sub_mask, LENSGB_FP64, s);
    if (launch_grad_rays(m->grid, m->st, n_inst, params, m->rec_d, m->coef_d, m->g_dcoef, gl,
                         area, m->g_partial, grad, m->grad_precision,
                         (unsigned char*)m->g_flag, m->grad_tau, s))
        return fail(LENSGB_ERR_CUDA, "gradient launch failed");
    return check_cuda("likelihood gradient launch");
}

static int ray_points(const lensgb_model* mc, const double* params, const double* x,
                      const double* y, double* bx, double* by, long long n, int want_alpha,
                      void* stream) {
    lensgb_model* m = const_cast<lensgb_model*>(mc);
    if (!m) return fail(LENSGB_ERR_INVALID, "null model");
    if (n < 0) return fail(LENSGB_ERR_INVALID, "negative point count");
    if (n == 0) return LENSGB_OK;
    if (!x || !y || !bx || !by) return fail(LENSGB_ERR_INVALID, "null coordinate pointer");
    if (!params && m->st.n_lens > 0) return fail(LENSGB_ERR_INVALID, "null params pointer");
    int rc = ensure_scratch(m, 1);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    // only the lens part of the row is meaningful; light records are unused
    StackDesc st = m->st;
    st.n_src = 0;
    st.n_ll = 0;
    launch_prepare(m->grid, st, params, 1, m->rec_d, m->rec_f, m->coef_d, m->coef_f, s);
    if ((rc = check_cuda("prepare launch"))) return rc;
    launch_ray_shoot_points(st, m->rec_d, m->coef_d, x, y, bx, by, n, want_alpha, s);
    return check_cuda("ray shooting launch");
}

int lensgb_ray_shooting(const lensgb_model* m, const double* params, const double* x,
                        const double* y, double* bx, double* by, long long n, void* stream) {
    return ray_points(m, params, x, y, bx, by, n, 0, stream);
}

int lensgb_alpha(const lensgb_model* m, const double* params, const double* x, const double* y,
                 double* ax, double* ay, long long n, void* stream) {
    return ray_points(m, params, x, y, ax, ay, n, 1, stream);
}

int lensgb_hessian(const lensgb_model* mc, const double* params, int n_inst, const double* x,
                   const double* y, double* out, long long n, void* stream) {
    lensgb_model* m = const_cast<lensgb_model*>(mc);
    if (!m) return fail(LENSGB_ERR_INVALID, "null model");
    if (n < 0 || n_inst < 0) return fail(LENSGB_ERR_INVALID, "negative point or system count");
    if (n == 0 || n_inst == 0) return LENSGB_OK;
    if (!x || !y || !out) return fail(LENSGB_ERR_INVALID, "null coordinate pointer");
    if (!params && m->st.n_lens > 0) return fail(LENSGB_ERR_INVALID, "null params pointer");
    if (!hessian_supported(m->st))
        return fail(LENSGB_ERR_UNSUPPORTED, "exact Hessians exist for EPL, SIE, NIE, NFW, TNFW, "
                                            "SHEAR and CONVERGENCE lenses");
    int rc = ensure_scratch(m, n_inst);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    StackDesc st = m->st;
    st.n_src = 0;
    st.n_ll = 0;
    launch_prepare(m->grid, st, params, n_inst, m->rec_d, m->rec_f, m->coef_d, m->coef_f, s);
    if ((rc = check_cuda("prepare launch"))) return rc;
    launch_hessian_points(st, m->rec_d, m->coef_d, params, x, y, out, n * n_inst, n, s);
    return check_cuda("hessian launch");
}

int lensgb_surface_brightness(const lensgb_model* mc, int which, const double* params,
                              const double* x, const double* y, double* out, long long n,
                              void* stream) {
    lensgb_model* m = const_cast<lensgb_model*>(mc);
    if (!m) return fail(LENSGB_ERR_INVALID, "null model");
    if (which != 0 && which != 1) return fail(LENSGB_ERR_INVALID, "which must be 0 or 1");
    if (n < 0) return fail(LENSGB_ERR_INVALID, "negative point count");
    if (n == 0) return LENSGB_OK;
    if (!x || !y || !out) return fail(LENSGB_ERR_INVALID, "null coordinate pointer");
    int rc = ensure_scratch(m, 1);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    // records for a row holding only this light model: offsets start at 0
    StackDesc st = m->st;
    st.n_lens = 0;
    const int base = which == 0 ? m->st.src_off[0] : m->st.ll_off[0];
    if (which == 0) {
        st.n_ll = 0;
        for (int k = 0; k < st.n_src; ++k) st.src_off[k] -= base;
    } else {
        st.n_src = 0;
        for (int k = 0; k < m->st.n_ll; ++k) {
            st.src[k] = m->st.ll[k];
            st.src_off[k] = m->st.ll_off[k] - base;
        }
        st.n_src = m->st.n_ll;
        st.n_ll = 0;
    }
    launch_prepare(m->grid, st, params, 1, m->rec_d, m->rec_f, m->coef_d, m->coef_f, s);
    if ((rc = check_cuda("prepare launch"))) return rc;
    launch_light_points(st, 0, m->rec_d, x, y, out, n, s);
    return check_cuda("surface brightness launch");
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Bulk handle: LensModelBulk / SinglePlaneBulk (lens_model_bulk.py:18-128,
// single_plane_bulk.py:20-131) with grow-only per-deflector scratch.
// ---------------------------------------------------------------------------
struct lensgb_bulk {
    BulkUnique u;
    int precision;
    double fp32_alpha_max = 0.05;
    bool need_coef = false;  // an EPL-type or NFW_ELLIPSE_CSE profile is in the list
    int cap = 0;
    int* tag = nullptr;
    double* rec_d = nullptr;
    float* rec_f = nullptr;
    double* coef_d = nullptr;
    float* coef_f = nullptr;
    float* pl_f = nullptr;    // multi-plane step table (8 floats per step)
    double* eps_d = nullptr;  // multi-plane, per step: FP32 T_cum / T_z - 1; FP64 1 / T_z (inv_tz_kernel)
};

static void bulk_free(lensgb_bulk* b) {
    cudaFree(b->tag);
    cudaFree(b->rec_d);
    cudaFree(b->rec_f);
    cudaFree(b->coef_d);
    cudaFree(b->coef_f);
    cudaFree(b->pl_f);
    cudaFree(b->eps_d);
    b->pl_f = nullptr;
    b->eps_d = nullptr;
    b->tag = nullptr;
    b->rec_d = nullptr;
    b->rec_f = nullptr;
    b->coef_d = nullptr;
    b->coef_f = nullptr;
    b->cap = 0;
}

static int bulk_ensure(lensgb_bulk* b, int n_defl) {
    if (n_defl <= b->cap) return LENSGB_OK;
    bulk_free(b);
    const size_t n = (size_t)n_defl;
    bool ok = cudaMalloc(&b->tag, n * sizeof(int)) == cudaSuccess &&
              cudaMalloc(&b->rec_d, n * REC_D * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&b->rec_f, n * REC_F * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&b->pl_f, n * 8 * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&b->eps_d, n * sizeof(double)) == cudaSuccess;
    if (ok && b->need_coef)
        ok = cudaMalloc(&b->coef_d, n * EPL_NMAX * sizeof(double)) == cudaSuccess &&
             cudaMalloc(&b->coef_f, n * EPL_NMAX * sizeof(float)) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        bulk_free(b);
        return fail(LENSGB_ERR_OOM, "bulk scratch allocation failed for " +
                                        std::to_string(n_defl) + " deflectors");
    }
    b->cap = n_defl;
    return LENSGB_OK;
}

extern "C" {

int lensgb_bulk_create(const int* codes, int n_unique, int precision, lensgb_bulk** out) {
    if (!out) return fail(LENSGB_ERR_INVALID, "null output handle pointer");
    *out = nullptr;
    if (n_unique < 0 || n_unique > LENSGB_BULK_MAX_UNIQUE)
        return fail(LENSGB_ERR_INVALID, "n_unique must be in [0, " +
                                            std::to_string(LENSGB_BULK_MAX_UNIQUE) + "]");
    if (n_unique > 0 && !codes) return fail(LENSGB_ERR_INVALID, "null unique code list");
    if (precision != LENSGB_FP64 && precision != LENSGB_FP32_SPLIT)
        return fail(LENSGB_ERR_UNSUPPORTED, "unknown precision " + std::to_string(precision));
    lensgb_bulk* b = new lensgb_bulk();
    b->u.n = n_unique;
    b->precision = precision;
    for (int k = 0; k < LENSGB_BULK_MAX_UNIQUE; ++k) b->u.code[k] = LENSGB_LENS_NULL;
    for (int k = 0; k < n_unique; ++k) {
        const int c = codes[k];
        if (c != LENSGB_LENS_NULL && lens_param_count(c) < 0) {
            delete b;
            return fail(LENSGB_ERR_UNSUPPORTED, "unknown lens profile code " + std::to_string(c));
        }
        b->u.code[k] = c;
        if (c == LENSGB_LENS_EPL || c == LENSGB_LENS_EPL_MULTIPOLE_M1M3M4 ||
            c == LENSGB_LENS_NFW_ELLIPSE_CSE)
            b->need_coef = true;
    }
    *out = b;
    return LENSGB_OK;
}

int lensgb_bulk_destroy(lensgb_bulk* b) {
    if (!b) return LENSGB_OK;
    bulk_free(b);
    delete b;
    return LENSGB_OK;
}

int lensgb_bulk_set_fp32_alpha_max(lensgb_bulk* b, double alpha_max) {
    if (!b) return fail(LENSGB_ERR_INVALID, "null bulk handle");
    if (!(alpha_max >= 0.0)) return fail(LENSGB_ERR_INVALID, "alpha_max must be >= 0");
    b->fp32_alpha_max = alpha_max;
    return LENSGB_OK;
}

int lensgb_bulk_ray_shooting(lensgb_bulk* b, const int* index, const double* params, int n_defl,
                             const double* x, const double* y, double* bx, double* by,
                             long long n, void* stream) {
    if (!b) return fail(LENSGB_ERR_INVALID, "null bulk handle");
    if (n_defl < 0) return fail(LENSGB_ERR_INVALID, "negative deflector count");
    if (n < 0) return fail(LENSGB_ERR_INVALID, "negative point count");
    if (n == 0) return LENSGB_OK;
    if (!x || !y || !bx || !by) return fail(LENSGB_ERR_INVALID, "null coordinate pointer");
    if (n_defl > 0 && (!index || !params))
        return fail(LENSGB_ERR_INVALID, "null index or params pointer");
    int rc = bulk_ensure(b, n_defl);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    launch_bulk_prepare(b->u, index, params, n_defl, b->fp32_alpha_max, b->tag, b->rec_d,
                        b->rec_f, b->coef_d, b->coef_f, s);
    if ((rc = check_cuda("bulk prepare launch"))) return rc;
    launch_bulk_ray_shooting(b->tag, b->rec_d, b->rec_f, b->coef_d, b->coef_f, n_defl, x, y, bx,
                             by, n, b->precision, s);
    return check_cuda("bulk ray shooting launch");
}

int lensgb_bulk_multi_plane_ray_shooting(lensgb_bulk* b, const int* index, const double* params,
                                         int n_steps, const double* T_ij, const double* T_z,
                                         const double* r2p, const double* alpha_x,
                                         const double* alpha_y, double* bx, double* by,
                                         long long n, void* stream) {
    if (!b) return fail(LENSGB_ERR_INVALID, "null bulk handle");
    if (n_steps < 1)
        return fail(LENSGB_ERR_INVALID, "multi-plane ray shooting needs at least one step "
                                        "(the source plane)");
    if (n < 0) return fail(LENSGB_ERR_INVALID, "negative point count");
    if (n == 0) return LENSGB_OK;
    if (!alpha_x || !alpha_y || !bx || !by)
        return fail(LENSGB_ERR_INVALID, "null coordinate pointer");
    if (!index || !params || !T_ij || !T_z || !r2p)
        return fail(LENSGB_ERR_INVALID, "null index, params or distance pointer");
    int rc = bulk_ensure(b, n_steps);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    launch_bulk_prepare(b->u, index, params, n_steps, b->fp32_alpha_max, b->tag, b->rec_d,
                        b->rec_f, b->coef_d, b->coef_f, s);
    if ((rc = check_cuda("bulk prepare launch"))) return rc;
    launch_multi_plane(b->tag, b->rec_d, b->rec_f, b->coef_d, b->coef_f, b->pl_f, b->eps_d, T_ij,
                       T_z, r2p, n_steps, alpha_x, alpha_y, bx, by, n, b->precision, s);
    return check_cuda("multi-plane ray shooting launch");
}

}  // extern "C"

// ---------------------------------------------------------------------------
// lensgb_image_noalloc: lensgb_image without any device allocation.
//
// Its scratch (per-profile records, EPL coefficient tables and the
// un-convolved image) lives in one fixed, file-scope device array of
// LENSGB_NOALLOC_SCRATCH_BYTES, which every GPU that loads this library holds
// until the process exits.  In host code `g_noalloc_scratch` names only a
// host-side stand-in, so its device address is looked up once per device with
// cudaGetSymbolAddress (on the first call made with that device current) and
// cached.  Every call overwrites each scratch element it later reads, so
// nothing has to be cleared between calls; calls that overlap on the GPU share
// the array and race.
// ---------------------------------------------------------------------------

#include <mutex>

static __device__ __align__(256) unsigned char g_noalloc_scratch[LENSGB_NOALLOC_SCRATCH_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
static void* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {nullptr};
static std::mutex g_noalloc_mutex;

static size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

static int noalloc_scratch_ptr(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return fail(LENSGB_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return fail(LENSGB_ERR_INVALID, "device ordinal out of range for the no-alloc scratch");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(LENSGB_ERR_CUDA, std::string("cudaGetSymbolAddress(no-alloc scratch): ") +
                                             cudaGetErrorString(e));
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return LENSGB_OK;
}

extern "C" int lensgb_image_noalloc(lensgb_model* m, const double* params, int n_inst,
                                    const void* psf, long long psf_stride, void* out, int flags,
                                    void* stream) {
    if (!m) return fail(LENSGB_ERR_INVALID, "null model");
    if (n_inst < 0 || n_inst > 65535)
        return fail(LENSGB_ERR_INVALID, "n_inst must be in 0..65535");
    if (n_inst == 0) return LENSGB_OK;
    if (!out || (!params && m->st.n_params > 0))
        return fail(LENSGB_ERR_INVALID, "null params or output pointer");
    const bool conv = !(flags & LENSGB_UNCONVOLVED) && m->desc.psf_type != LENSGB_PSF_NONE;
    if (conv && !psf) return fail(LENSGB_ERR_INVALID, "null PSF kernel pointer");
    if (psf_stride < 0) return fail(LENSGB_ERR_INVALID, "negative PSF stride");
    if ((conv && m->hr_conv) || m->sub)
        return fail(LENSGB_ERR_UNSUPPORTED,
                    "lensgb_image_noalloc does not provide supersampled convolution or "
                    "sub-frames");
    const int n_prof = m->st.n_lens + m->st.n_src + m->st.n_ll;
    const size_t nrec = (size_t)n_inst * (n_prof > 0 ? n_prof : 1);
    const size_t ncoef = (size_t)n_inst * (m->st.n_epl > 0 ? m->st.n_epl : 1) * EPL_NMAX;
    const size_t esz = m->desc.precision == LENSGB_FP64 ? 8 : 4;
    const size_t b_rec_d = align256(nrec * REC_D * sizeof(double));
    const size_t b_rec_f = align256(nrec * REC_F * sizeof(float));
    const size_t b_coef_d = align256(ncoef * sizeof(double));
    const size_t b_coef_f = align256(ncoef * sizeof(float));
    const size_t b_low = conv ? align256((size_t)n_inst * m->grid.nx * m->grid.ny * esz) : 0;
    const bool fp32 = m->desc.precision == LENSGB_FP32_SPLIT;
    const size_t b_list = fp32 ? align256((size_t)n_inst * m->grid.nx * m->grid.ny * 4) : 0;
    const size_t b_cnt = fp32 ? 256 : 0;
    const size_t need = b_rec_d + b_rec_f + b_coef_d + b_coef_f + b_low + b_list + b_cnt;
    if (need > (size_t)LENSGB_NOALLOC_SCRATCH_BYTES) {
        char msg[256];
        snprintf(msg, sizeof msg,
                 "this call needs %zu bytes of scratch; lensgb_image_noalloc holds at most %zu "
                 "bytes (use fewer systems per call, or lensgb_image)",
                 need, (size_t)LENSGB_NOALLOC_SCRATCH_BYTES);
        return fail(LENSGB_ERR_INVALID, msg);
    }
    int rc = check_refine_size(m, n_inst);
    if (rc) return rc;
    void* base = nullptr;
    rc = noalloc_scratch_ptr(&base);
    if (rc) return rc;
    unsigned char* p = (unsigned char*)base;
    double* rec_d = (double*)p;
    float* rec_f = (float*)(p + b_rec_d);
    double* coef_d = (double*)(p + b_rec_d + b_rec_f);
    float* coef_f = (float*)(p + b_rec_d + b_rec_f + b_coef_d);
    void* low = p + b_rec_d + b_rec_f + b_coef_d + b_coef_f;
    unsigned int* list = fp32 ? (unsigned int*)((unsigned char*)low + b_low) : nullptr;
    unsigned int* cnt = fp32 ? (unsigned int*)((unsigned char*)low + b_low + b_list) : nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    launch_prepare(m->grid, m->st, params, n_inst, rec_d, rec_f, coef_d, coef_f, s);
    if ((rc = check_cuda("prepare launch"))) return rc;
    const double scale = m->pixel_width * m->pixel_width;
    RefineArgs rf = refine_args(m, n_inst, list, cnt);
    if (rf.tau > 0.f && cudaMemsetAsync(cnt, 0, sizeof(unsigned int), s) != cudaSuccess)
        return check_cuda("refine counter reset");
    launch_raytrace(m->grid, m->st, n_inst, rec_d, rec_f, coef_d, coef_f, conv ? low : out, flags,
                    scale, m->desc.precision, rf, s, nullptr, 0, tuned_ppt(m, n_inst));
    if ((rc = check_cuda("raytrace launch"))) return rc;
    if (conv) {
        if (launch_conv(low, out, psf, psf_stride, n_inst, m->grid.ny, m->grid.nx,
                        m->desc.kernel_size, m->desc.psf_type == LENSGB_PSF_GAUSSIAN ? 1 : 0,
                        m->desc.precision, s, m->tune_rows))
            return fail(LENSGB_ERR_CUDA, "convolution shared-memory configuration failed");
        if ((rc = check_cuda("convolution launch"))) return rc;
    }
    return LENSGB_OK;
}
