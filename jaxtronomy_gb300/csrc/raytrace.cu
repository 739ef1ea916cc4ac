// Fused ray-tracing kernel: for every supersampled ray of every system,
// deflection sum -> lensed source light -> lens light, then the s x s block
// mean into the (ny, nx) pixel image.  The ray grid exists only in registers
// and one shared-memory staging buffer; the image leaves the kernel already
// multiplied by pixel_width^2 and flux_scaling.
//
// Mapping: blockIdx.y = system; blockIdx.x = a run of P consecutive pixels
// (row-major).  Each thread owns one supersampled ray per pass over the
// CTA's P*s^2 rays; consecutive threads own neighbouring sub-rays, so warps
// stay spatially coherent.
//
// Reference path (JAXtronomy source tree):
//   ray grid          ImSim/Numerics/grid.py:48-72 (lenstronomy make_subgrid)
//   deflection sum    LensModel/single_plane.py:39-56,113-139
//   source mapping    ImSim/image_model.py:347-354 (lenstronomy Image2SourceMapping)
//   light sum         LightModel/light_model_base.py:230-252
//   re-binning        ImSim/Numerics/grid.py:102-117, Util/image_util.py:79-98
//   pixel area        ImSim/Numerics/numerics.py:177
#include "launch.h"
#include "profiles.cuh"

namespace lensgb {

template <typename R>
struct RayCtx {
    // FP64: absolute ray coordinate; FP32: exact/small parts of the offset
    // from supersampled ray (0,0)
    double X, Y;
    float px, lx, py, ly;
};

template <typename R>
__device__ __forceinline__ void ray_offset(const RayCtx<R>& c, const R* rec, R& dx, R& dy) {
    if (sizeof(R) == 8) {
        dx = (R)(c.X - (double)rec[RD_CX]);
        dy = (R)(c.Y - (double)rec[RD_CY]);
    } else {
        const float* fr = (const float*)rec;
        dx = (R)split_offset(fr[RF_X0H], fr[RF_X0L], c.px, c.lx);
        dy = (R)split_offset(fr[RF_Y0H], fr[RF_Y0L], c.py, c.ly);
    }
}

template <typename R>
__device__ __forceinline__ void lens_deflect(int code, const R* rec, const R* F, R dx, R dy, R& ax,
                                             R& ay) {
    switch (code) {
        case LENSGB_LENS_SIE:
        case LENSGB_LENS_NIE: nie_deflect<R>(rec, dx, dy, ax, ay); break;
        case LENSGB_LENS_EPL: epl_deflect<R>(rec, F, dx, dy, ax, ay); break;
        case LENSGB_LENS_SHEAR: shear_deflect<R>(rec, dx, dy, ax, ay); break;
        case LENSGB_LENS_NFW: nfw_deflect<R>(rec, dx, dy, ax, ay); break;
        case LENSGB_LENS_TNFW: tnfw_deflect<R>(rec, dx, dy, ax, ay); break;
        default: ax = 0; ay = 0; break;
    }
}

template <typename R>
__device__ __forceinline__ R ray_flux(const GridDesc& g, const StackDesc& st, const R* srec,
                                      const R* scoef, int recw, int I, int J, int flags) {
    RayCtx<R> c;
    if (sizeof(R) == 8) {
        c.X = g.ra00 + (double)J * g.ax + (double)I * g.bx;
        c.Y = g.dec00 + (double)J * g.ay + (double)I * g.by;
    } else {
        float fJ = (float)J, fI = (float)I;
        c.px = fJ * g.ax_hi + fI * g.bx_hi;
        c.lx = fJ * g.ax_lo + fI * g.bx_lo;
        c.py = fJ * g.ay_hi + fI * g.by_hi;
        c.ly = fJ * g.ay_lo + fI * g.by_lo;
    }
    R flux = 0;
    const bool do_src = !(flags & LENSGB_NO_SOURCE) && st.n_src > 0;
    if (do_src) {
        R axs = 0, ays = 0;
        for (int p = 0; p < st.n_lens; ++p) {
            const R* rec = srec + p * recw;
            R dx, dy, ax, ay;
            ray_offset<R>(c, rec, dx, dy);
            const int es = st.epl_slot[p];
            lens_deflect<R>(st.lens[p], rec, es >= 0 ? scoef + es * EPL_NMAX : nullptr, dx, dy, ax,
                            ay);
            axs += ax;
            ays += ay;
        }
        axs *= (R)st.alpha_scaling;
        ays *= (R)st.alpha_scaling;
        R fs = 0;
        for (int k = 0; k < st.n_src; ++k) {
            const R* rec = srec + (st.n_lens + k) * recw;
            const R sc = (R)st.src_scale[k];
            R dx, dy;
            if (sizeof(R) == 8) {
                // beta = theta - scale * alpha, then the profile shift
                double bxv = c.X - (double)(sc * axs);
                double byv = c.Y - (double)(sc * ays);
                dx = (R)(bxv - (double)rec[RD_CX]);
                dy = (R)(byv - (double)rec[RD_CY]);
            } else {
                ray_offset<R>(c, rec, dx, dy);
                dx -= sc * axs;
                dy -= sc * ays;
            }
            fs += sersic_flux<R>(rec, dx, dy);
        }
        flux += fs;
    }
    if (!(flags & LENSGB_NO_LENS_LIGHT)) {
        R fl = 0;
        for (int k = 0; k < st.n_ll; ++k) {
            const R* rec = srec + (st.n_lens + st.n_src + k) * recw;
            R dx, dy;
            ray_offset<R>(c, rec, dx, dy);
            fl += sersic_flux<R>(rec, dx, dy);
        }
        flux += fl;
    }
    return flux * (R)st.flux_scaling;
}

template <typename R>
__global__ void __launch_bounds__(256)
raytrace_kernel(GridDesc g, StackDesc st, int P, const R* __restrict__ rec, const R* __restrict__ coef,
                R* __restrict__ out, int flags, double out_scale) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int recw = sizeof(R) == 8 ? REC_D : REC_F;
    const int n_prof = st.n_lens + st.n_src + st.n_ll;
    const int inst = blockIdx.y;
    const int s = g.s, s2 = s * s;
    R* srec = (R*)smem_raw;
    R* scoef = srec + n_prof * recw;
    R* sbuf = scoef + st.n_epl * EPL_NMAX;

    const R* grec = rec + (long long)inst * n_prof * recw;
    for (int k = threadIdx.x; k < n_prof * recw; k += blockDim.x) srec[k] = grec[k];
    __syncthreads();
    for (int p = 0; p < st.n_lens; ++p) {
        const int es = st.epl_slot[p];
        if (es < 0) continue;
        const int nmax = (int)srec[p * recw + slot<R>(8)];
        const R* gc = coef + ((long long)inst * st.n_epl + es) * EPL_NMAX;
        for (int k = threadIdx.x; k < nmax; k += blockDim.x) scoef[es * EPL_NMAX + k] = gc[k];
    }
    __syncthreads();

    const long long npix = (long long)g.nx * g.ny;
    const long long pix0 = (long long)blockIdx.x * P;
    const int nray = P * s2;
    for (int r = threadIdx.x; r < nray; r += blockDim.x) {
        const int p = r / s2, sub = r - p * s2;
        const long long pix = pix0 + p;
        R v = 0;
        if (pix < npix) {
            const int row = (int)(pix / g.nx), col = (int)(pix - (long long)row * g.nx);
            const int si = sub / s, sj = sub - si * s;
            v = ray_flux<R>(g, st, srec, scoef, recw, row * s + si, col * s + sj, flags);
        }
        sbuf[r] = v;
    }
    __syncthreads();
    R* o = out + (long long)inst * npix;
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        const long long pix = pix0 + p;
        if (pix >= npix) break;
        const R* b = sbuf + p * s2;
        R acc = 0;
        if (s == 1) {
            acc = b[0];
        } else {
            // mean over sub-columns, then over sub-rows (image_util.py:93)
            for (int si = 0; si < s; ++si) {
                R rs = 0;
                for (int sj = 0; sj < s; ++sj) rs += b[si * s + sj];
                acc += rs / (R)s;
            }
            acc = acc / (R)s;
        }
        o[pix] = acc * (R)out_scale;
    }
}

static int g_num_sms = 0;

int launch_raytrace(const GridDesc& g, const StackDesc& st, int n_inst, const double* rec_d,
                    const float* rec_f, const double* coef_d, const float* coef_f, void* out,
                    int flags, double out_scale, int precision, cudaStream_t stream) {
    if (g_num_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_num_sms <= 0) g_num_sms = 152;
    }
    const int threads = 256;
    const int s2 = g.s * g.s;
    const long long npix = (long long)g.nx * g.ny;
    // rays per thread: enough CTAs to fill the GPU several times, at most 9
    long long rays = npix * s2 * (long long)n_inst;
    long long target = (long long)g_num_sms * 8 * threads;
    int rpt = (int)((rays + target - 1) / target);
    rpt = rpt < 1 ? 1 : (rpt > 9 ? 9 : rpt);
    int P = (rpt * threads) / s2;
    if (P < 1) P = 1;
    const int n_prof = st.n_lens + st.n_src + st.n_ll;
    const int esz = precision == LENSGB_FP64 ? 8 : 4;
    const int recw = precision == LENSGB_FP64 ? REC_D : REC_F;
    size_t smem = (size_t)(n_prof * recw + st.n_epl * EPL_NMAX + P * s2) * esz;
    dim3 grid((unsigned)((npix + P - 1) / P), (unsigned)n_inst);
    if (precision == LENSGB_FP64) {
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(raytrace_kernel<double>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        raytrace_kernel<double><<<grid, threads, smem, stream>>>(g, st, P, rec_d, coef_d,
                                                                 (double*)out, flags, out_scale);
    } else {
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(raytrace_kernel<float>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        raytrace_kernel<float><<<grid, threads, smem, stream>>>(g, st, P, rec_f, coef_f,
                                                                (float*)out, flags, out_scale);
    }
    return 0;
}

}  // namespace lensgb
