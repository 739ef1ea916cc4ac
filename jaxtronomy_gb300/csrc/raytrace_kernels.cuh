// Fused ray-tracing kernels: for every supersampled ray of every system,
// deflection sum -> lensed source light -> lens light, then the s x s block
// mean into the (ny, nx) pixel image.  The ray grid exists only in registers;
// the image leaves the kernel already multiplied by pixel_width^2 and
// flux_scaling.
//
// Mapping: blockIdx.y = system; each thread owns the s^2 supersampled rays of
// one pixel at a time (pixels of a CTA are consecutive in row-major order, so
// a warp covers 32 neighbouring pixels of a row and stays spatially coherent).
// Profile records of the CTA's system sit in shared memory.
//
// FP32 path ("FP32 split"): the bulk arithmetic is FP32.  Coordinate offsets
// from every profile centre are formed with FP64 accuracy (split_offset), and
// each sub-ray predicts the relative error its FP32 deflection causes in the
// source light (Sersic log-gradient x the FP32 error bound of beta = theta -
// alpha, weighted by the source's share of the ray's flux).  Pixels where the
// prediction exceeds `tau` -- rays landing close to a steep source centre,
// where the lens equation cancels theta against alpha -- are appended to a
// list that refine_kernel recomputes in FP64 with the code of the FP64 path.
//
// Reference path (JAXtronomy source tree):
//   ray grid          ImSim/Numerics/grid.py:48-72 (lenstronomy make_subgrid)
//   deflection sum    LensModel/single_plane.py:39-56,113-139
//   source mapping    ImSim/image_model.py:347-354 (lenstronomy Image2SourceMapping)
//   light sum         LightModel/light_model_base.py:230-252
//   re-binning        ImSim/Numerics/grid.py:102-117, Util/image_util.py:79-98
//   pixel area        ImSim/Numerics/numerics.py:177
#pragma once

#include <type_traits>

#include "launch.h"
#include "profiles.cuh"
#include "raytrace_variants.h"

namespace lensgb {

// Lens-stack selector: C0/C1 are compile-time lens codes (0 = absent); C0 =
// GENERIC (-1, raytrace_variants.h) selects the kernel that walks the runtime stack.

// Offsets of the pixel's base ray (sub-ray 0, 0) from one profile centre.
struct PixOff {
    float bx, by;  // FP32 path: FP64-accurate offset of the base ray, rounded once
};

// FP32 base-ray offset of pixel (row, col) from the centre of record rec.
__device__ __forceinline__ PixOff pix_offset_f(const GridDesc& g, const float* rec, float Jb,
                                               float Ib) {
    PixOff o;
    o.bx = split_offset(rec[RF_X0H], rec[RF_X0L], Jb * g.ax_hi + Ib * g.bx_hi,
                        Jb * g.ax_lo + Ib * g.bx_lo);
    o.by = split_offset(rec[RF_Y0H], rec[RF_Y0L], Jb * g.ay_hi + Ib * g.by_hi,
                        Jb * g.ay_lo + Ib * g.by_lo);
    return o;
}

// Compile-time profile count helpers
template <int C0, int C1>
struct LensStackT {
    static constexpr bool generic = (C0 == GENERIC);
    static constexpr int n = generic ? 0 : ((C0 > 0) + (C1 > 0));
    __host__ __device__ static constexpr int code(int i) { return i == 0 ? C0 : C1; }
};

// FP64 flux of one supersampled ray (I, J): the FP64 path and the refine pass.
template <int C0, int C1, int NS, int NLL>
__device__ __forceinline__ double ray_flux_d(const GridDesc& g, const StackDesc& st,
                                             const double* srec, const double* scoef, int I,
                                             int J, int flags) {
    using LS = LensStackT<C0, C1>;
    const double X = g.ra00 + (double)J * g.ax + (double)I * g.bx;
    const double Y = g.dec00 + (double)J * g.ay + (double)I * g.by;
    const int n_lens = LS::generic ? st.n_lens : LS::n;
    const int n_src = NS >= 0 ? NS : st.n_src;
    const int n_ll = NLL >= 0 ? NLL : st.n_ll;
    double flux = 0;
    if (!(flags & LENSGB_NO_SOURCE) && n_src > 0) {
        double axs = 0, ays = 0;
#pragma unroll (LS::generic ? 1 : 8)
        for (int p = 0; p < (LS::generic ? MAX_PROF : LS::n); ++p) {
            if (p >= n_lens) break;
            const double* rec = srec + p * REC_D;
            const int code = LS::generic ? st.lens[p] : LS::code(p);
            const int es = st.epl_slot[p];
            double ax, ay;
            lens_deflect<double>(code, rec, es >= 0 ? scoef + es * EPL_NMAX : nullptr,
                                 X - rec[RD_CX], Y - rec[RD_CY], ax, ay);
            axs += ax;
            ays += ay;
        }
        axs *= st.alpha_scaling;
        ays *= st.alpha_scaling;
        double fs = 0;
#pragma unroll (LS::generic ? 1 : 8)
        for (int k = 0; k < (NS >= 0 ? NS : MAX_PROF); ++k) {
            if (k >= n_src) break;
            const double* rec = srec + (n_lens + k) * REC_D;
            const double sc = st.src_scale[k];
            // beta = theta - scale * alpha, then the profile shift
            const double bxv = X - sc * axs, byv = Y - sc * ays;
            fs += sersic_flux<double>(rec, bxv - rec[RD_CX], byv - rec[RD_CY]);
        }
        flux += fs;
    }
    if (!(flags & LENSGB_NO_LENS_LIGHT)) {
        double fl = 0;
#pragma unroll (LS::generic ? 1 : 8)
        for (int k = 0; k < (NLL >= 0 ? NLL : MAX_PROF); ++k) {
            if (k >= n_ll) break;
            const double* rec = srec + (n_lens + n_src + k) * REC_D;
            fl += sersic_flux<double>(rec, X - rec[RD_CX], Y - rec[RD_CY]);
        }
        flux += fl;
    }
    return flux * st.flux_scaling;
}

// Flux of one supersampled ray for the FP32 path's refine pass: the ray, the
// deflections and beta in FP64 (beta = theta - alpha is what cancels in FP32),
// then each light profile in FP32 (sersic_f, the FP32 kernel's own arithmetic)
// from its FP64 offset rounded once.  The Sersic evaluations are most of the
// FP64 ray's work, and their FP32 rounding (~1e-7 relative here) is far below
// the FP32 path's bar; only the cancelling difference needs FP64.
template <int C0, int C1, int NS, int NLL>
__device__ __forceinline__ double ray_flux_refine(const GridDesc& g, const StackDesc& st,
                                                  const double* srec, const double* scoef,
                                                  const float* frec, int I, int J, int flags) {
    using LS = LensStackT<C0, C1>;
    const double X = g.ra00 + (double)J * g.ax + (double)I * g.bx;
    const double Y = g.dec00 + (double)J * g.ay + (double)I * g.by;
    const int n_lens = LS::generic ? st.n_lens : LS::n;
    const int n_src = NS >= 0 ? NS : st.n_src;
    const int n_ll = NLL >= 0 ? NLL : st.n_ll;
    double flux = 0;
    if (!(flags & LENSGB_NO_SOURCE) && n_src > 0) {
        double axs = 0, ays = 0;
#pragma unroll (LS::generic ? 1 : 8)
        for (int p = 0; p < (LS::generic ? MAX_PROF : LS::n); ++p) {
            if (p >= n_lens) break;
            const double* rec = srec + p * REC_D;
            const int code = LS::generic ? st.lens[p] : LS::code(p);
            const int es = st.epl_slot[p];
            double ax, ay;
            lens_deflect<double>(code, rec, es >= 0 ? scoef + es * EPL_NMAX : nullptr,
                                 X - rec[RD_CX], Y - rec[RD_CY], ax, ay);
            axs += ax;
            ays += ay;
        }
        axs *= st.alpha_scaling;
        ays *= st.alpha_scaling;
        float fs = 0.f;
#pragma unroll (LS::generic ? 1 : 8)
        for (int k = 0; k < (NS >= 0 ? NS : MAX_PROF); ++k) {
            if (k >= n_src) break;
            const double* rec = srec + (n_lens + k) * REC_D;
            const double sc = st.src_scale[k];
            const double bxv = X - sc * axs, byv = Y - sc * ays;
            float gk;
            fs += sersic_f<false>(frec + (n_lens + k) * REC_F, (float)(bxv - rec[RD_CX]),
                                  (float)(byv - rec[RD_CY]), gk);
        }
        flux += (double)fs;
    }
    if (!(flags & LENSGB_NO_LENS_LIGHT)) {
        float fl = 0.f;
#pragma unroll (LS::generic ? 1 : 8)
        for (int k = 0; k < (NLL >= 0 ? NLL : MAX_PROF); ++k) {
            if (k >= n_ll) break;
            const double* rec = srec + (n_lens + n_src + k) * REC_D;
            float gk;
            fl += sersic_f<false>(frec + (n_lens + n_src + k) * REC_F, (float)(X - rec[RD_CX]),
                                  (float)(Y - rec[RD_CY]), gk);
        }
        flux += (double)fl;
    }
    return flux * st.flux_scaling;
}

// FP64 value of pixel (row, col): mean over sub-columns then sub-rows
// (image_util.py:93), times out_scale.
template <int C0, int C1, int NS, int NLL>
__device__ __forceinline__ double pixel_value_d(const GridDesc& g, const StackDesc& st,
                                                const double* srec, const double* scoef, int row,
                                                int col, int flags, double out_scale) {
    const int s = g.s;
    double acc = 0;
    for (int si = 0; si < s; ++si) {
        double rs = 0;
        for (int sj = 0; sj < s; ++sj)
            rs += ray_flux_d<C0, C1, NS, NLL>(g, st, srec, scoef, row * s + si, col * s + sj, flags);
        acc += s == 1 ? rs : rs / (double)s;
    }
    if (s > 1) acc = acc / (double)s;
    return acc * out_scale;
}

// Load the CTA's system records (and EPL tables) into shared memory.
template <typename R>
__device__ __forceinline__ void load_records(const StackDesc& st, const R* rec, const R* coef,
                                             int inst, R* srec, R* scoef) {
    const int recw = sizeof(R) == 8 ? REC_D : REC_F;
    const int n_prof = st.n_lens + st.n_src + st.n_ll;
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
}

// ---------------------------------------------------------------------------
// FP64 kernel
// ---------------------------------------------------------------------------
template <int C0, int C1, int NS, int NLL>
__global__ void __launch_bounds__(256)
raytrace_fp64_kernel(GridDesc g0, StackDesc st, int ppt, const double* __restrict__ rec,
                     const double* __restrict__ coef, double* __restrict__ out, int flags,
                     double out_scale, MixedTab mt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n_prof = st.n_lens + st.n_src + st.n_ll;
    double* srec = (double*)smem_raw;
    double* scoef = srec + n_prof * REC_D;
    // uniform launch: one pass for (system blockIdx.y, tile blockIdx.x);
    // mixed launch: grid-stride loop over every system's tiles
    const bool mixed = mt.grid != nullptr;
    const int n_grp = mixed ? *mt.count : 0;
    const int n_tiles = mixed ? __ldg(mt.tile_off + n_grp) : 1;
    for (int t = mixed ? (int)blockIdx.x : 0; t < n_tiles; t += mixed ? (int)gridDim.x : 1) {
        int inst = blockIdx.y, tile = blockIdx.x;
        if (mixed) {
            const int j = find_segment(mt.tile_off, n_grp, t);
            inst = __ldg(mt.sys + j);
            tile = t - __ldg(mt.tile_off + j);
        }
        const GridDesc g = mixed ? mt.grid[inst] : g0;
        const double osc = mixed ? mt.scale[inst] : out_scale;
        load_records<double>(st, rec, coef, inst, srec, scoef);
        const long long npix = (long long)g.nx * g.ny;
        double* o = out + (mixed ? mt.off[inst] : (long long)inst * npix);
        const long long base = (long long)tile * blockDim.x * ppt;
        for (int k = 0; k < ppt; ++k) {
            const long long pix = base + (long long)k * blockDim.x + threadIdx.x;
            if (pix >= npix) break;
            const int row = (int)(pix / g.nx), col = (int)(pix - (long long)row * g.nx);
            o[pix] = pixel_value_d<C0, C1, NS, NLL>(g, st, srec, scoef, row, col, flags, osc);
        }
        if (mixed) __syncthreads();  // before the next tile reloads the records
    }
}

// FP64 kernel for launches too small to fill the GPU with one thread per
// pixel (one system of 180x180 pixels is 127 CTAs of 256 pixel-threads on 152
// SMs): one thread per supersampled ray.  A CTA takes RAY_PIX = 256 / s^2
// consecutive pixels of one system, its threads trace their ray into shared
// memory, and the first RAY_PIX threads combine each pixel's s^2 fluxes in the
// order of pixel_value_d -- the same ray_flux_d code and the same sums, so a
// pixel equals the one-thread-per-pixel kernel's value bit for bit.
template <int C0, int C1, int NS, int NLL>
__global__ void __launch_bounds__(256)
raytrace_fp64_rays_kernel(GridDesc g, StackDesc st, const double* __restrict__ rec,
                          const double* __restrict__ coef, double* __restrict__ out, int flags,
                          double out_scale) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n_prof = st.n_lens + st.n_src + st.n_ll;
    double* srec = (double*)smem_raw;
    double* scoef = srec + n_prof * REC_D;
    double* sub = scoef + st.n_epl * EPL_NMAX;  // 256 ray fluxes
    const int inst = blockIdx.y;
    load_records<double>(st, rec, coef, inst, srec, scoef);
    const int s = g.s, s2 = s * s;
    const int per = 256 / s2;
    const long long npix = (long long)g.nx * g.ny;
    const long long pix0 = (long long)blockIdx.x * per;
    const int t = threadIdx.x;
    const int el = t / s2, k = t - el * s2;
    double v = 0.0;
    if (el < per && pix0 + el < npix) {
        const long long pix = pix0 + el;
        const int row = (int)(pix / g.nx), col = (int)(pix - (long long)row * g.nx);
        const int si = k / s, sj = k - si * s;
        v = ray_flux_d<C0, C1, NS, NLL>(g, st, srec, scoef, row * s + si, col * s + sj, flags);
    }
    sub[t] = v;
    __syncthreads();
    if (t < per && pix0 + t < npix) {
        const double* b = sub + t * s2;
        double acc = 0;
        for (int si = 0; si < s; ++si) {
            double rs = 0;
            for (int sj = 0; sj < s; ++sj) rs += b[si * s + sj];
            acc += s == 1 ? rs : rs / (double)s;
        }
        if (s > 1) acc = acc / (double)s;
        out[(long long)inst * npix + pix0 + t] = acc * out_scale;
    }
}

// ---------------------------------------------------------------------------
// FP32 kernel (pass 1)
// ---------------------------------------------------------------------------

// SS > 0 fixes the supersampling factor at compile time (the sub-ray loops
// unroll); SS = 0 reads it from the grid.
template <int C0, int C1, int NS, int NLL, int SS, bool MIXED>
__global__ void __launch_bounds__(256)
raytrace_fp32_kernel(GridDesc g0, StackDesc st, int ppt, const float* __restrict__ rec,
                     const float* __restrict__ coef, float* __restrict__ out, int flags,
                     float out_scale, RefineArgs rf, MixedTab mt) {
    using LS = LensStackT<C0, C1>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n_prof = st.n_lens + st.n_src + st.n_ll;
    float* srec = (float*)smem_raw;
    float* scoef = srec + n_prof * REC_F;
    constexpr bool mixed = MIXED;  // compile-time, so a uniform launch reads g0 directly
    // uniform launch: one pass for (system blockIdx.y, tile blockIdx.x);
    // mixed launch: grid-stride loop over every system's tiles of 256 pixels
    const int n_grp = mixed ? *mt.count : 0;
    const int n_tiles = mixed ? __ldg(mt.tile_off + n_grp) : 1;
    for (int t = mixed ? (int)blockIdx.x : 0; t < n_tiles; t += mixed ? (int)gridDim.x : 1) {
        int inst = blockIdx.y, tile = blockIdx.x;
        if (mixed) {
            const int j = find_segment(mt.tile_off, n_grp, t);
            inst = __ldg(mt.sys + j);
            tile = t - __ldg(mt.tile_off + j);
            out_scale = (float)mt.scale[inst];
        }
        const GridDesc& g = mixed ? mt.grid[inst] : g0;
        load_records<float>(st, rec, coef, inst, srec, scoef);

        const int n_lens = LS::generic ? st.n_lens : LS::n;
        const int n_src = NS >= 0 ? NS : st.n_src;
        const int n_ll = NLL >= 0 ? NLL : st.n_ll;
        constexpr int ML = LS::generic ? MAX_PROF : (LS::n > 0 ? LS::n : 1);
        constexpr int MS = NS >= 0 ? (NS > 0 ? NS : 1) : MAX_PROF;
        constexpr int MLL = NLL >= 0 ? (NLL > 0 ? NLL : 1) : MAX_PROF;
        // compile-time stacks keep every record in registers for the whole CTA
        constexpr int NPC = LS::generic ? 1 : LS::n + MS + MLL;
        float lr[NPC][REC_F];
        if (!LS::generic) {
#pragma unroll
            for (int i = 0; i < NPC; ++i)
#pragma unroll
                for (int k = 0; k < REC_F; ++k)
                    lr[i][k] = i < n_prof ? srec[i * REC_F + k] : 0.f;
        }
#define REC(i) (LS::generic ? srec + (i) * REC_F : lr[(i)])
        const bool do_src = !(flags & LENSGB_NO_SOURCE) && n_src > 0;
        const bool do_ll = !(flags & LENSGB_NO_LENS_LIGHT) && n_ll > 0;
        const bool refine = rf.tau > 0.f && do_src;
        const int s = SS > 0 ? SS : g.s;
        const float inv_s = 1.f / (float)s;
        const float axf = g.ax_hi + g.ax_lo, bxf = g.bx_hi + g.bx_lo;
        const float ayf = g.ay_hi + g.ay_lo, byf = g.by_hi + g.by_lo;
        const long long npix = (long long)g.nx * g.ny;
        const long long img0 = mixed ? mt.off[inst] : (long long)inst * npix;
        float* o = out + img0;
        const long long base = (long long)tile * blockDim.x * ppt;

        for (int kk = 0; kk < ppt; ++kk) {
            const long long pix = base + (long long)kk * blockDim.x + threadIdx.x;
            if (pix >= npix) break;
            // pixel index of one system (< 2^31): 32-bit division
            const unsigned int p32 = (unsigned int)pix;
            const int row = (int)(p32 / (unsigned int)g.nx), col = (int)(p32 - (unsigned int)row * g.nx);
            const float Jb = (float)(col * s), Ib = (float)(row * s);
            // base-ray offsets from every profile centre, FP64-accurate
            PixOff ol[ML], os[MS], oll[MLL];
#pragma unroll (LS::generic ? 1 : 8)
            for (int p = 0; p < ML; ++p)
                if (p < n_lens && do_src) ol[p] = pix_offset_f(g, REC(p), Jb, Ib);
#pragma unroll (LS::generic ? 1 : 8)
            for (int k = 0; k < MS; ++k)
                if (k < n_src && do_src) os[k] = pix_offset_f(g, REC(n_lens + k), Jb, Ib);
#pragma unroll (LS::generic ? 1 : 8)
            for (int k = 0; k < MLL; ++k)
                if (k < n_ll && do_ll) oll[k] = pix_offset_f(g, REC(n_lens + n_src + k), Jb, Ib);

            float acc = 0.f;
            bool flag = false;
#pragma unroll (SS > 0 ? SS : 1)
            for (int si = 0; si < (SS > 0 ? SS : s); ++si) {
                float rs = 0.f;
                const float fi = (float)si;
                // compile-time stack and supersampling: the row's SS sub-rays are
                // deflected together (lens_deflect_row_f), in the same per-ray
                // order of profiles as the per-ray loop below
                constexpr bool ROW = SS > 0 && !LS::generic;
                constexpr int NRW = ROW ? SS : 1;
                float rax[NRW], ray_[NRW];
                if constexpr (ROW) {
                    if (do_src) {
#pragma unroll
                        for (int sj = 0; sj < NRW; ++sj) rax[sj] = ray_[sj] = 0.f;
#pragma unroll
                        for (int p = 0; p < ML; ++p) {
                            if (p >= n_lens) break;
                            const int es = st.epl_slot[p];
                            float dxr[NRW], dyr[NRW], axr[NRW], ayr[NRW];
#pragma unroll
                            for (int sj = 0; sj < NRW; ++sj) {
                                const float fj = (float)sj;
                                dxr[sj] = ol[p].bx + fmaf(fi, bxf, fj * axf);
                                dyr[sj] = ol[p].by + fmaf(fi, byf, fj * ayf);
                            }
                            lens_deflect_row_f<NRW>(LS::code(p), REC(p),
                                                    es >= 0 ? scoef + es * EPL_NMAX : nullptr, dxr,
                                                    dyr, axr, ayr);
#pragma unroll
                            for (int sj = 0; sj < NRW; ++sj) {
                                rax[sj] += axr[sj];
                                ray_[sj] += ayr[sj];
                            }
                        }
                    }
                }
#pragma unroll (SS > 0 ? SS : 1)
                for (int sj = 0; sj < (SS > 0 ? SS : s); ++sj) {
                    // sub-ray displacement from the base ray: below one pixel, so a
                    // plain FP32 product keeps an absolute error of ~1e-9 pixel
                    const float fj = (float)sj;
                    const float ddx = fmaf(fi, bxf, fj * axf);
                    const float ddy = fmaf(fi, byf, fj * ayf);
                    float flux = 0.f;
                    if (do_src) {
                        float axs = 0.f, ays = 0.f;
                        if constexpr (ROW) {
                            axs = rax[sj];
                            ays = ray_[sj];
                        } else {
#pragma unroll (LS::generic ? 1 : 8)
                            for (int p = 0; p < ML; ++p) {
                                if (p >= n_lens) break;
                                const int code = LS::generic ? st.lens[p] : LS::code(p);
                                const int es = st.epl_slot[p];
                                float ax, ay;
                                lens_deflect<float>(code, REC(p),
                                                    es >= 0 ? scoef + es * EPL_NMAX : nullptr,
                                                    ol[p].bx + ddx, ol[p].by + ddy, ax, ay);
                                axs += ax;
                                ays += ay;
                            }
                        }
                        // alpha_scaling is folded into each source's scale (and
                        // its magnitude into the refine predictor's kappa)
                        float fsrc = 0.f, gsum = 0.f;
#pragma unroll (LS::generic ? 1 : 8)
                        for (int k = 0; k < MS; ++k) {
                            if (k >= n_src) break;
                            const float sc = st.src_scale_f[k];
                            const float sca = sc * st.alpha_scaling_f;
                            float gk;
                            const float fk = sersic_flux_grad(REC(n_lens + k), os[k].bx + ddx - sca * axs,
                                                              os[k].by + ddy - sca * ays, gk);
                            fsrc += fk;
                            gsum += fk * gk * sc;
                        }
                        flux = fsrc;
                        if (do_ll) {
#pragma unroll (LS::generic ? 1 : 8)
                            for (int k = 0; k < MLL; ++k) {
                                if (k >= n_ll) break;
                                flux += sersic_flux<float>(REC(n_lens + n_src + k), oll[k].bx + ddx,
                                                           oll[k].by + ddy);
                            }
                        }
                        if (refine) {
                            // predicted relative error of this ray's flux from the FP32
                            // error of beta (kappa * |alpha|) through the source gradients
                            const float dbeta = (rf.kappa * fabsf(st.alpha_scaling_f)) *
                                                (fabsf(axs) + fabsf(ays));
                            flag |= gsum * dbeta > rf.tau * flux;
                        }
                    } else if (do_ll) {
#pragma unroll (LS::generic ? 1 : 8)
                        for (int k = 0; k < MLL; ++k) {
                            if (k >= n_ll) break;
                            flux += sersic_flux<float>(REC(n_lens + n_src + k), oll[k].bx + ddx,
                                                       oll[k].by + ddy);
                        }
                    }
                    rs += flux;
                }
                acc += s == 1 ? rs : rs * inv_s;
            }
            if (s > 1) acc *= inv_s;
            o[pix] = acc * st.flux_scaling_f * out_scale;
            if (flag) {
                const unsigned int slot_i = atomicAdd(rf.count, 1u);
                rf.list[slot_i] = (unsigned int)(img0 + pix);
            }
        }
        if (mixed) __syncthreads();  // before the next tile reloads the records
    }
#undef REC
}

// ---------------------------------------------------------------------------
// Refine pass: recompute the listed pixels with FP64 rays, deflections and
// beta (ray_flux_refine; records read from global memory).
// ---------------------------------------------------------------------------
// One thread per (listed pixel, sub-ray); the s^2 sub-ray fluxes of a pixel are
// combined in shared memory in the order of pixel_value_d.
constexpr int REFINE_THREADS = 128;

template <int C0, int C1, int NS, int NLL>
__global__ void __launch_bounds__(REFINE_THREADS)
refine_kernel(GridDesc g, StackDesc st, const double* __restrict__ rec,
              const double* __restrict__ coef, const float* __restrict__ frec,
              float* __restrict__ out, int flags, double out_scale, RefineArgs rf) {
    __shared__ double sub[32 * 32];  // s <= 32
    const unsigned int n = *rf.count;
    const int n_prof = st.n_lens + st.n_src + st.n_ll;
    const int s = g.s, s2 = s * s;
    const int per = s2 <= REFINE_THREADS ? REFINE_THREADS / s2 : 1;  // pixels per chunk
    for (unsigned int first = blockIdx.x * per; first < n; first += gridDim.x * per) {
        for (int w = threadIdx.x; w < per * s2; w += REFINE_THREADS) {
            const int el = w / s2, k = w - el * s2;
            double v = 0.0;
            if (first + el < n) {
                const long long e = (long long)rf.list[first + el];
                const int inst = (int)(e / ((long long)g.nx * g.ny));
                const long long pix = e - (long long)inst * g.nx * g.ny;
                const int row = (int)(pix / g.nx), col = (int)(pix - (long long)row * g.nx);
                const int si = k / s, sj = k - si * s;
                v = ray_flux_refine<C0, C1, NS, NLL>(
                    g, st, rec + (long long)inst * n_prof * REC_D,
                    coef + (long long)inst * st.n_epl * EPL_NMAX,
                    frec + (long long)inst * n_prof * REC_F, row * s + si, col * s + sj, flags);
            }
            sub[w] = v;
        }
        __syncthreads();
        for (int el = threadIdx.x; el < per; el += REFINE_THREADS) {
            if (first + el >= n) break;
            const double* b = sub + el * s2;
            double acc = 0;
            for (int si = 0; si < s; ++si) {
                double rs = 0;
                for (int sj = 0; sj < s; ++sj) rs += b[si * s + sj];
                acc += s == 1 ? rs : rs / (double)s;
            }
            if (s > 1) acc = acc / (double)s;
            out[rf.list[first + el]] = (float)(acc * out_scale);
        }
        __syncthreads();
    }
}

// Refine pass of a mixed launch (systems of different grids and supersampling
// factors): one warp per listed pixel, its lanes evaluating the pixel's s^2
// sub-rays (system s from the pixel's grid), combined by lane 0 in the order
// of pixel_value_d.
template <int C0, int C1, int NS, int NLL>
__global__ void __launch_bounds__(REFINE_THREADS)
refine_mixed_kernel(StackDesc st, const double* __restrict__ rec,
                    const double* __restrict__ coef, const float* __restrict__ frec,
                    float* __restrict__ out, int flags, RefineArgs rf, MixedTab mt) {
    constexpr int WARPS = REFINE_THREADS / 32;
    __shared__ double sub[WARPS][32 * 32];  // s <= 32
    const unsigned int n = *rf.count;
    const int n_prof = st.n_lens + st.n_src + st.n_ll;
    const int n_mixed = *mt.n_inst;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (unsigned int i = blockIdx.x * WARPS + warp; i < n; i += gridDim.x * WARPS) {
        const long long e = (long long)rf.list[i];
        // the system whose image holds element e: off[inst] <= e < off[inst + 1]
        int lo = 0, hi = n_mixed - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (mt.off[mid] <= e) lo = mid; else hi = mid - 1;
        }
        const GridDesc g = mt.grid[lo];
        const int s = g.s, s2 = s * s;
        const long long pix = e - mt.off[lo];
        const int row = (int)(pix / g.nx), col = (int)(pix - (long long)row * g.nx);
        const double* r = rec + (long long)lo * n_prof * REC_D;
        const double* cf = coef + (long long)lo * st.n_epl * EPL_NMAX;
        for (int k = lane; k < s2; k += 32) {
            const int si = k / s, sj = k - si * s;
            sub[warp][k] = ray_flux_refine<C0, C1, NS, NLL>(
                g, st, r, cf, frec + (long long)lo * n_prof * REC_F, row * s + si, col * s + sj,
                flags);
        }
        __syncwarp();
        if (lane == 0) {
            const double* b = sub[warp];
            double acc = 0;
            for (int si = 0; si < s; ++si) {
                double rs = 0;
                for (int sj = 0; sj < s; ++sj) rs += b[si * s + sj];
                acc += s == 1 ? rs : rs / (double)s;
            }
            if (s > 1) acc = acc / (double)s;
            out[e] = (float)(acc * mt.scale[lo]);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
template <int C0, int C1, int NS, int NLL>
void launch_variant(const GridDesc& g, const StackDesc& st, int n_inst, const double* rec_d,
                           const float* rec_f, const double* coef_d, const float* coef_f,
                           void* out, int flags, double out_scale, int precision,
                           const RefineArgs& rf, const MixedTab& mt, int mixed_ctas,
                           int ppt_override, cudaStream_t stream) {
    const int threads = 256;
    const long long npix = (long long)g.nx * g.ny;
    // pixels per thread: enough CTAs to fill the GPU several times over
    long long target = (long long)num_sms() * 8 * threads;
    long long total = npix * (long long)n_inst;
    int ppt = (int)((total + target - 1) / target);
    ppt = ppt < 1 ? 1 : (ppt > 8 ? 8 : ppt);
    if (ppt_override > 0) ppt = ppt_override;  // a tuned choice (lensgb_model_autotune)
    if (mt.grid) ppt = 1;  // mixed launches: one tile of 256 pixels per CTA
    const long long per_cta = (long long)threads * ppt;
    dim3 grid = mt.grid ? dim3((unsigned)mixed_ctas, 1)
                        : dim3((unsigned)((npix + per_cta - 1) / per_cta), (unsigned)n_inst);
    const int n_prof = st.n_lens + st.n_src + st.n_ll;
    if (precision == LENSGB_FP64) {
        size_t smem = (size_t)(n_prof * REC_D + st.n_epl * EPL_NMAX) * sizeof(double);
        // one thread per ray when one thread per pixel leaves the GPU under-filled
        // (fewer than 4 CTAs per SM) and a CTA holds at least one pixel's rays
        const long long pix_ctas = (long long)grid.x * grid.y;
        if (!mt.grid && ppt_override <= 0 && g.s * g.s <= 256 &&
            pix_ctas < 4LL * num_sms()) {
            const int per = 256 / (g.s * g.s);
            const dim3 rgrid((unsigned)((npix + per - 1) / per), (unsigned)n_inst);
            const size_t rsmem = smem + 256 * sizeof(double);
            if (rsmem > 48 * 1024)
                cudaFuncSetAttribute(raytrace_fp64_rays_kernel<C0, C1, NS, NLL>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsmem);
            raytrace_fp64_rays_kernel<C0, C1, NS, NLL><<<rgrid, 256, rsmem, stream>>>(
                g, st, rec_d, coef_d, (double*)out, flags, out_scale);
            return;
        }
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(raytrace_fp64_kernel<C0, C1, NS, NLL>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        raytrace_fp64_kernel<C0, C1, NS, NLL><<<grid, threads, smem, stream>>>(
            g, st, ppt, rec_d, coef_d, (double*)out, flags, out_scale, mt);
    } else {
        size_t smem = (size_t)(n_prof * REC_F + st.n_epl * EPL_NMAX) * sizeof(float);
        // compile-time supersampling factor for the specialised stacks
        auto run = [&](auto ss_tag) {
            constexpr int SS = decltype(ss_tag)::value;
            if (mt.grid) {
                if (smem > 48 * 1024)
                    cudaFuncSetAttribute(raytrace_fp32_kernel<C0, C1, NS, NLL, SS, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                raytrace_fp32_kernel<C0, C1, NS, NLL, SS, true><<<grid, threads, smem, stream>>>(
                    g, st, ppt, rec_f, coef_f, (float*)out, flags, (float)out_scale, rf, mt);
            } else {
                if (smem > 48 * 1024)
                    cudaFuncSetAttribute(raytrace_fp32_kernel<C0, C1, NS, NLL, SS, false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                raytrace_fp32_kernel<C0, C1, NS, NLL, SS, false><<<grid, threads, smem, stream>>>(
                    g, st, ppt, rec_f, coef_f, (float*)out, flags, (float)out_scale, rf, mt);
            }
        };
        // a mixed launch runs its supersampling group's kernel (group 0: the
        // run-time-s kernel, which reads s from each system's grid)
        const int ss = mt.grid ? mt.s_group : g.s;
        if (C0 == GENERIC) run(std::integral_constant<int, 0>());
        else if (ss == 1) run(std::integral_constant<int, 1>());
        else if (ss == 2) run(std::integral_constant<int, 2>());
        else if (ss == 3) run(std::integral_constant<int, 3>());
        else if (ss == 4) run(std::integral_constant<int, 4>());
        else run(std::integral_constant<int, 0>());
        if (rf.tau > 0.f && !(flags & LENSGB_NO_SOURCE) && st.n_src > 0 && mt.refine) {
            const int rblocks = num_sms() * 4;
            if (mt.grid)
                refine_mixed_kernel<C0, C1, NS, NLL><<<rblocks, REFINE_THREADS, 0, stream>>>(
                    st, rec_d, coef_d, rec_f, (float*)out, flags, rf, mt);
            else
                refine_kernel<C0, C1, NS, NLL><<<rblocks, REFINE_THREADS, 0, stream>>>(
                    g, st, rec_d, coef_d, rec_f, (float*)out, flags, out_scale, rf);
        }
    }
}

}  // namespace lensgb
