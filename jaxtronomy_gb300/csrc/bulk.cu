// Many-deflector ray shooting: SinglePlaneBulk.ray_shooting
// (JAXtronomy LensModel/single_plane_bulk.py:109-131), beta = x - sum_i alpha_i.
//
// The reference materialises an [n_deflectors, n_rays] FP64 array through
// lax.map + lax.switch and sums it.  Here one thread owns one ray and walks
// the deflector list; the block stages the FP32 records and tags of 64
// deflectors at a time in shared memory, so every thread of a warp evaluates
// the same deflector (the profile switch is warp-uniform); each thread carries
// two rays, so every staged record serves two evaluations.  In FP32_SPLIT
// mode a deflector tagged FP32 is evaluated from the split centre
// (x_hi - c_hi) + (x_lo - c_lo) and summed in FP32 within the chunk; chunk
// sums and FP64-tagged terms accumulate in FP64.
#include "launch.h"
#include "profiles.cuh"

namespace lensgb {

// Launch shapes (compile-time; -D overrides serve shape sweeps).
#ifndef LENSGB_BULK_RPT
#define LENSGB_BULK_RPT 2
#endif
#ifndef LENSGB_MP_RPT
#define LENSGB_MP_RPT 3
#endif
#ifndef LENSGB_MP_MAXNREG
#define LENSGB_MP_MAXNREG 160
#endif
#ifndef LENSGB_MP_THREADS
#define LENSGB_MP_THREADS 128
#endif
constexpr int BULK_CHUNK = 64;
constexpr int BULK_THREADS = 256;
constexpr int BULK_RPT = LENSGB_BULK_RPT;  // rays per thread (i, i + BULK_THREADS, ...)

template <bool F32>
__global__ void __launch_bounds__(BULK_THREADS)
bulk_ray_kernel(const int* __restrict__ tag, const double* __restrict__ rec_d,
                const float* __restrict__ rec_f, const double* __restrict__ coef_d,
                const float* __restrict__ coef_f, int n_defl, const double* __restrict__ x,
                const double* __restrict__ y, double* __restrict__ bx, double* __restrict__ by,
                long long n) {
    __shared__ __align__(16) float srec[BULK_CHUNK * REC_F];
    __shared__ int stag[BULK_CHUNK];
    const long long i0 = (long long)blockIdx.x * (BULK_THREADS * BULK_RPT) + threadIdx.x;
    // FP64: the ray in FP64.  FP32_SPLIT: the ray as an FP32 pair only (hi + lo
    // equals it to 2^-48 relative), fenced so that the loop never rebuilds the
    // pair from an FP64 value in FP64 arithmetic.
    double xd[BULK_RPT], yd[BULK_RPT], axd[BULK_RPT], ayd[BULK_RPT];
    float xh[BULK_RPT], xl[BULK_RPT], yh[BULK_RPT], yl[BULK_RPT];
#pragma unroll
    for (int k = 0; k < BULK_RPT; ++k) {
        const long long i = i0 + (long long)k * BULK_THREADS;
        xd[k] = i < n ? x[i] : 0.0;
        yd[k] = i < n ? y[i] : 0.0;
        split_double(xd[k], xh[k], xl[k]);
        split_double(yd[k], yh[k], yl[k]);
        if (F32) {
            asm volatile("" : "+f"(xh[k]), "+f"(xl[k]), "+f"(yh[k]), "+f"(yl[k]));
            xd[k] = (double)xh[k] + (double)xl[k];
            yd[k] = (double)yh[k] + (double)yl[k];
        }
        axd[k] = 0.0;
        ayd[k] = 0.0;
    }
    // An FP32 TNFW subhalo: the rays' polynomials as straight-line code, then the
    // closed form for rays inside x = max(tau, 1); sums into (sx, sy).
    auto tnfw_rays = [&](const float* rf, float* sx, float* sy) {
        const float ch = rf[RF_X0H], cl = rf[RF_X0L], dh = rf[RF_Y0H], dl = rf[RF_Y0L];
        float dx[BULK_RPT], dy[BULK_RPT], ax[BULK_RPT], ay[BULK_RPT];
        bool in[BULK_RPT], any = false;
#pragma unroll
        for (int k = 0; k < BULK_RPT; ++k) {
            dx[k] = __fadd_rn(__fsub_rn(xh[k], ch), __fsub_rn(xl[k], cl));
            dy[k] = __fadd_rn(__fsub_rn(yh[k], dh), __fsub_rn(yl[k], dl));
            in[k] = tnfw_far_f(rf, dx[k], dy[k], ax[k], ay[k]);
            any |= in[k];
        }
        if (any) {
#pragma unroll
            for (int k = 0; k < BULK_RPT; ++k)
                if (in[k]) tnfw_near_f(rf, dx[k], dy[k], ax[k], ay[k]);
        }
#pragma unroll
        for (int k = 0; k < BULK_RPT; ++k) {
            sx[k] += ax[k];
            sy[k] += ay[k];
        }
    };
    for (int c0 = 0; c0 < n_defl; c0 += BULK_CHUNK) {
        const int cnt = n_defl - c0 < BULK_CHUNK ? n_defl - c0 : BULK_CHUNK;
        __syncthreads();
        if (F32) {
            const float* src = rec_f + (long long)c0 * REC_F;
            for (int k = threadIdx.x; k < cnt * REC_F; k += blockDim.x) srec[k] = src[k];
        }
        for (int k = threadIdx.x; k < cnt; k += blockDim.x) stag[k] = tag[c0 + k];
        __syncthreads();
        float sx[BULK_RPT], sy[BULK_RPT];
#pragma unroll
        for (int k = 0; k < BULK_RPT; ++k) sx[k] = sy[k] = 0.f;
        for (int j = 0; j < cnt; ++j) {
            const int t = stag[j];
            if (F32 && t == LENSGB_LENS_TNFW) {
                // the common deflector (an FP32 subhalo), decided by one comparison
                tnfw_rays(srec + j * REC_F, sx, sy);
                continue;
            }
            const int code = t & BULK_CODE_MASK;
            if (code == LENSGB_LENS_NULL) continue;
            const long long g = c0 + j;
            if (!F32 || (t & BULK_TAG_FP64)) {
                const double* rd = rec_d + g * REC_D;
                const double* cd = coef_d ? coef_d + g * EPL_NMAX : nullptr;
#pragma unroll
                for (int k = 0; k < BULK_RPT; ++k) {
                    const double xk = F32 ? (double)xh[k] + (double)xl[k] : xd[k];
                    const double yk = F32 ? (double)yh[k] + (double)yl[k] : yd[k];
                    double ax, ay;
                    lens_deflect<double>(code, rd, cd, xk - rd[RD_CX], yk - rd[RD_CY], ax, ay);
                    axd[k] += ax;
                    ayd[k] += ay;
                }
            } else {
                const float* rf = srec + j * REC_F;
                const float ch = rf[RF_X0H], cl = rf[RF_X0L], dh = rf[RF_Y0H], dl = rf[RF_Y0L];
                if (code == LENSGB_LENS_TNFW) {
                    tnfw_rays(rf, sx, sy);
                } else {
                    const float* cf = coef_f ? coef_f + g * EPL_NMAX : nullptr;
#pragma unroll
                    for (int k = 0; k < BULK_RPT; ++k) {
                        const float dx = __fadd_rn(__fsub_rn(xh[k], ch), __fsub_rn(xl[k], cl));
                        const float dy = __fadd_rn(__fsub_rn(yh[k], dh), __fsub_rn(yl[k], dl));
                        float ax, ay;
                        lens_deflect<float>(code, rf, cf, dx, dy, ax, ay);
                        sx[k] += ax;
                        sy[k] += ay;
                    }
                }
            }
        }
#pragma unroll
        for (int k = 0; k < BULK_RPT; ++k) {
            axd[k] += (double)sx[k];
            ayd[k] += (double)sy[k];
        }
    }
#pragma unroll
    for (int k = 0; k < BULK_RPT; ++k) {
        const long long i = i0 + (long long)k * BULK_THREADS;
        if (i < n) {
            const double xk = F32 ? (double)xh[k] + (double)xl[k] : xd[k];
            const double yk = F32 ? (double)yh[k] + (double)yl[k] : yd[k];
            bx[i] = xk - axd[k];
            by[i] = yk - ayd[k];
        }
    }
}

// ---------------------------------------------------------------------------
// Multi-plane ray shooting: MultiPlaneBulk.ray_shooting
// (JAXtronomy LensModel/MultiPlane/multi_plane_bulk.py:152-200).  The
// reference scans the deflectors in redshift order with the carry
// (alpha, x): x += alpha T_ij[i]; alpha -= r2p[i] alpha_i(x / T_z[i]);
// beta = x / T_z[last].
//
// FP64 follows that recurrence step by step (x / T_z as x times a per-step
// 1 / T_z).  FP32_SPLIT writes it as
//   alpha = theta - v,  x = theta T_cum - d,
//   v += r2p_i alpha_i,  d += v T_ij[i]  (T_cum = running sum of T_ij),
// so that the ray state is the small deflection v and the displacement d,
// carried as FP32 pairs (h + l), next to the FP64 start angle theta.  The
// offset to deflector centre c at plane i is then
//   x / T_z - c = (theta - c) + theta eps_i - d / T_z[i],  eps_i = T_cum/T_z - 1,
// with (theta - c) taken from the FP64-accurate (hi, lo) splits.  Consecutive
// deflectors with T_ij = 0 and equal T_z and r2p share one plane: their
// deflections are evaluated at the same position (as in the reference, where
// x does not move between them) and summed before the plane's r2p scales them
// into v.  FP32-tagged terms are summed in FP32 per plane; CONVERGENCE (linear
// in the offset) is evaluated as an FP32-pair product and FP64-tagged terms in
// FP64 from an FP64 offset, both summed as FP32 pairs.
// ---------------------------------------------------------------------------
constexpr int MP_THREADS = LENSGB_MP_THREADS;
constexpr int MP_RPT = LENSGB_MP_RPT;
constexpr int MP_CHUNK = 64;
constexpr int PL_F = 8;  // per-step floats: dT hi/lo, 1/T_z hi/lo, eps, r2p hi/lo, tag bits

// 16-byte asynchronous global -> shared copy (sm_80+ cp.async, L2 only) and its
// group fences; the wait is the hardware's wait on this thread's own copies.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned a = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(a), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Plane table of n_steps steps, one CTA of PREP_THREADS per PREP_THREADS steps:
// pl_f receives the FP32 step constants and the step's tag with
// BULK_TAG_PLANE where a new plane starts, eps_d the FP64 eps.  Each CTA sums
// the T_ij before its steps itself (T_cum needs only ~1e-16 relative accuracy:
// it enters eps, a correction to the ray offset).
constexpr int PREP_THREADS = 64;

__global__ void __launch_bounds__(PREP_THREADS)
plane_prepare_kernel(const double* __restrict__ dT, const double* __restrict__ Tz,
                     const double* __restrict__ r2p, int n_steps, const int* __restrict__ tag,
                     float* __restrict__ pl_f, double* __restrict__ eps_d) {
    __shared__ double sc[PREP_THREADS];
    const int t = threadIdx.x;
    const int i0 = blockIdx.x * PREP_THREADS;
    const int i = i0 + t;
    double acc = 0.0;
    for (int k = t; k < i0; k += PREP_THREADS) acc += dT[k];
    sc[t] = acc;
    __syncthreads();
    for (int w = PREP_THREADS / 2; w > 0; w >>= 1) {
        if (t < w) sc[t] += sc[t + w];
        __syncthreads();
    }
    const double before = sc[0];
    __syncthreads();
    // inclusive scan of this CTA's T_ij (Hillis-Steele)
    sc[t] = i < n_steps ? dT[i] : 0.0;
    __syncthreads();
    for (int w = 1; w < PREP_THREADS; w <<= 1) {
        const double v = t >= w ? sc[t - w] : 0.0;
        __syncthreads();
        sc[t] += v;
        __syncthreads();
    }
    if (i >= n_steps) return;
    const double cum = before + sc[t];
    const bool start = i == 0 || dT[i] != 0.0 || Tz[i] != Tz[i - 1] || r2p[i] != r2p[i - 1];
    const int tg = tag[i] | (start ? BULK_TAG_PLANE : 0);
    const double e = cum / Tz[i] - 1.0;
    eps_d[i] = e;
    float* f = pl_f + (long long)i * PL_F;
    split_double(dT[i], f[0], f[1]);
    split_double(1.0 / Tz[i], f[2], f[3]);
    f[4] = (float)e;
    split_double(r2p[i], f[5], f[6]);
    f[7] = __int_as_float(tg);
}

// (h, l) += (bh, bl) for FP32 pairs with |l| << |h|.
__device__ __forceinline__ void pair_add(float& h, float& l, float bh, float bl) {
    float e;
    const float s = two_sum(h, bh, e);
    e = __fadd_rn(e, __fadd_rn(l, bl));
    h = __fadd_rn(s, e);
    l = __fsub_rn(e, __fsub_rn(h, s));
}

// (ph, pl) = (ah, al) * (bh, bl), to about 2^-44 relative.
__device__ __forceinline__ void pair_mul(float ah, float al, float bh, float bl, float& ph,
                                         float& pl) {
    ph = __fmul_rn(ah, bh);
    pl = __fmaf_rn(ah, bh, -ph);
    pl = __fmaf_rn(ah, bl, __fmaf_rn(al, bh, pl));
}

// 3 rays per thread, 160 registers and 128 threads: a 400^2-ray call (417
// CTAs) is resident in one wave at 3 CTAs per SM with no spills; fewer
// registers made the compiler rebuild ray state in FP64 or spill.  Launch-shape
// sweep on GB300 (400^2 rays, 5501 steps): 128 threads 2.32 ms, 96 2.37, 64
// 2.41, 192 2.51, 32 3.16, 256 3.69 (two CTAs on some SMs, one on others);
// 4 rays / 168 registers 2.74, 2 rays / 128 registers 3.08.
template <bool F32>
__global__ void __maxnreg__(LENSGB_MP_MAXNREG)
multi_plane_kernel(const int* __restrict__ tag, const double* __restrict__ rec_d,
                   const float* __restrict__ rec_f, const double* __restrict__ coef_d,
                   const float* __restrict__ coef_f, const float* __restrict__ pl_f,
                   const double* __restrict__ eps_d, const double* __restrict__ dT,
                   const double* __restrict__ Tz, const double* __restrict__ r2p, int n_steps,
                   const double* __restrict__ ax0, const double* __restrict__ ay0,
                   double* __restrict__ bx, double* __restrict__ by, long long n) {
    // FP32_SPLIT: two chunk buffers of records and step tables, the next chunk
    // copied asynchronously while the current one is evaluated; FP64: tags only
    constexpr int NBUF = F32 ? 2 : 1;
    __shared__ __align__(16) float srec_b[NBUF][F32 ? MP_CHUNK * REC_F : 4];
    __shared__ __align__(16) float spl_b[NBUF][F32 ? MP_CHUNK * PL_F : 4];
    __shared__ int stag[MP_CHUNK];
    const long long i0 = (long long)blockIdx.x * (MP_THREADS * MP_RPT) + threadIdx.x;
    auto issue_chunk = [&](int c0, int buf) {
        const int cnt = n_steps - c0 < MP_CHUNK ? n_steps - c0 : MP_CHUNK;
        const float* src = rec_f + (long long)c0 * REC_F;
        for (int k = threadIdx.x; k < cnt * (REC_F / 4); k += blockDim.x)
            cp_async16(&srec_b[buf][4 * k], src + 4 * k);
        const float* ps = pl_f + (long long)c0 * PL_F;
        for (int k = threadIdx.x; k < cnt * (PL_F / 4); k += blockDim.x)
            cp_async16(&spl_b[buf][4 * k], ps + 4 * k);
        cp_async_commit();
    };
    // FP64 state: x (position) and alpha.  FP32_SPLIT state: the start angle theta
    // as an FP32 pair (tH + tL equals theta to 2^-48 relative), v, d, the plane's
    // pending sums and lc = tL + the plane's offset correction (folded once per
    // plane, so an offset costs three additions) -- no FP64 value stays live
    // through the loop, so none of it is recomputed there in FP64.
    double xs[2][MP_RPT], al[2][MP_RPT];
    float tH[2][MP_RPT], tL[2][MP_RPT], vh[2][MP_RPT], vl[2][MP_RPT], dh[2][MP_RPT],
        dl[2][MP_RPT], ph[2][MP_RPT], pq[2][MP_RPT], s32[2][MP_RPT], lc[2][MP_RPT];
#pragma unroll
    for (int k = 0; k < MP_RPT; ++k) {
        const long long i = i0 + (long long)k * MP_THREADS;
        const double th[2] = {i < n ? ax0[i] : 0.0, i < n ? ay0[i] : 0.0};
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            xs[c][k] = 0.0;
            al[c][k] = th[c];
            split_double(th[c], tH[c][k], tL[c][k]);
            // opaque to the optimiser: kept as registers, never rebuilt from theta
            asm volatile("" : "+f"(tH[c][k]), "+f"(tL[c][k]));
            vh[c][k] = vl[c][k] = dh[c][k] = dl[c][k] = 0.f;
            ph[c][k] = pq[c][k] = s32[c][k] = 0.f;
            lc[c][k] = tL[c][k];
        }
    }
    float rh = 0.f, rl = 0.f;  // the current plane's r2p
    // An FP32 TNFW step: the rays' polynomials as straight-line code, then the
    // closed form for rays inside x = max(tau, 1); sums into s32.
    auto tnfw_rays = [&](const float* rf, const float* ox, const float* oy) {
        float ax[MP_RPT], ay[MP_RPT];
        bool in[MP_RPT], any = false;
#pragma unroll
        for (int k = 0; k < MP_RPT; ++k) {
            in[k] = tnfw_far_f<true>(rf, ox[k], oy[k], ax[k], ay[k]);
            any |= in[k];
        }
        if (any) {
#pragma unroll
            for (int k = 0; k < MP_RPT; ++k)
                if (in[k]) tnfw_near_f(rf, ox[k], oy[k], ax[k], ay[k]);
        }
#pragma unroll
        for (int k = 0; k < MP_RPT; ++k) {
            s32[0][k] += ax[k];
            s32[1][k] += ay[k];
        }
    };
    // FP32 offsets of the rays from deflector record rf's split centre
    auto offsets = [&](const float* rf, float* ox, float* oy) {
        const float ch = rf[RF_X0H], cl = rf[RF_X0L], dh0 = rf[RF_Y0H], dl0 = rf[RF_Y0L];
#pragma unroll
        for (int k = 0; k < MP_RPT; ++k) {
            ox[k] = __fadd_rn(__fsub_rn(tH[0][k], ch), __fsub_rn(lc[0][k], cl));
            oy[k] = __fadd_rn(__fsub_rn(tH[1][k], dh0), __fsub_rn(lc[1][k], dl0));
        }
    };
    if (F32) issue_chunk(0, 0);
    for (int c0 = 0, it = 0; c0 < n_steps; c0 += MP_CHUNK, ++it) {
        const int cnt = n_steps - c0 < MP_CHUNK ? n_steps - c0 : MP_CHUNK;
        const int buf = F32 ? (it & 1) : 0;
        const float* srec = srec_b[buf];
        const float* spl = spl_b[buf];
        if (F32) {
            // every thread finished the chunk before last, whose buffer the next
            // copy overwrites (the barrier at the end of the previous iteration)
            if (c0 + MP_CHUNK < n_steps) {
                issue_chunk(c0 + MP_CHUNK, buf ^ 1);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
        } else {
            for (int k = threadIdx.x; k < cnt; k += blockDim.x) stag[k] = tag[c0 + k];
        }
        __syncthreads();
        for (int j = 0; j < cnt; ++j) {
            const int t = F32 ? __float_as_int(spl[j * PL_F + 7]) : stag[j];
            if (F32 && t == LENSGB_LENS_TNFW) {
                // the common step (an FP32 subhalo inside the current plane),
                // decided by one comparison
                float ox[MP_RPT], oy[MP_RPT];
                offsets(srec + j * REC_F, ox, oy);
                tnfw_rays(srec + j * REC_F, ox, oy);
                continue;
            }
            const int code = t & BULK_CODE_MASK;
            const long long g = c0 + j;
            if (!F32) {
                // reference recurrence (multi_plane_bulk.py:181-194)
                const double dt = dT[g];
#pragma unroll
                for (int k = 0; k < MP_RPT; ++k) {
                    xs[0][k] += al[0][k] * dt;
                    xs[1][k] += al[1][k] * dt;
                }
                if (code == LENSGB_LENS_NULL) continue;
                // x / T_z as x * (1 / T_z): within an ulp of the division
                const double itz = eps_d[g], r = r2p[g];
                const double* rd = rec_d + g * REC_D;
                const double* cd = coef_d ? coef_d + g * EPL_NMAX : nullptr;
#pragma unroll
                for (int k = 0; k < MP_RPT; ++k) {
                    double ax, ay;
                    lens_deflect<double>(code, rd, cd, xs[0][k] * itz - rd[RD_CX],
                                         xs[1][k] * itz - rd[RD_CY], ax, ay);
                    al[0][k] -= ax * r;
                    al[1][k] -= ay * r;
                }
                continue;
            }
            if (t & BULK_TAG_PLANE) {
                const float* pl = spl + j * PL_F;
#pragma unroll
                for (int k = 0; k < MP_RPT; ++k) {
#pragma unroll
                    for (int c = 0; c < 2; ++c) {
                        // flush the previous plane: v += r2p * (pending + FP32 sum)
                        float e;
                        const float sh = two_sum(ph[c][k], s32[c][k], e);
                        const float sl = __fadd_rn(pq[c][k], e);
                        float qh, ql;
                        pair_mul(sh, sl, rh, rl, qh, ql);
                        pair_add(vh[c][k], vl[c][k], qh, ql);
                        ph[c][k] = pq[c][k] = s32[c][k] = 0.f;
                        // d += v * T_ij
                        pair_mul(vh[c][k], vl[c][k], pl[0], pl[1], qh, ql);
                        pair_add(dh[c][k], dl[c][k], qh, ql);
                        // theta eps - d / T_z
                        const float disp =
                            __fmaf_rn(dh[c][k], pl[2], __fmaf_rn(dh[c][k], pl[3],
                                                                 __fmul_rn(dl[c][k], pl[2])));
                        lc[c][k] = __fadd_rn(tL[c][k], __fmaf_rn(tH[c][k], pl[4], -disp));
                    }
                }
                rh = pl[5];
                rl = pl[6];
            }
            if (code == LENSGB_LENS_NULL) continue;
            const float* rf = srec + j * REC_F;
            if (code == LENSGB_LENS_CONVERGENCE) {
                const float kh = rf[slot<float>(2)], kl = rf[slot<float>(3)];
                const float ch[2] = {rf[RF_X0H], rf[RF_Y0H]}, cl[2] = {rf[RF_X0L], rf[RF_Y0L]};
#pragma unroll
                for (int k = 0; k < MP_RPT; ++k) {
#pragma unroll
                    for (int c = 0; c < 2; ++c) {
                        float e;
                        const float a = two_sum(tH[c][k], -ch[c], e);
                        const float b = __fsub_rn(lc[c][k], cl[c]);
                        float e2;
                        const float xh = two_sum(a, __fadd_rn(e, b), e2);
                        float qh, ql;
                        pair_mul(xh, e2, kh, kl, qh, ql);
                        pair_add(ph[c][k], pq[c][k], qh, ql);
                    }
                }
            } else if (t & BULK_TAG_FP64) {
                const double* rd = rec_d + g * REC_D;
                const double* cd = coef_d ? coef_d + g * EPL_NMAX : nullptr;
                // 1 / T_z from the step table's FP32 pair (to ~2^-48 relative), so
                // no FP64 division runs per deflector
                const float* pl = spl + j * PL_F;
                const double ep = eps_d[g], itz = (double)pl[2] + (double)pl[3];
#pragma unroll
                for (int k = 0; k < MP_RPT; ++k) {
                    double o[2];
#pragma unroll
                    for (int c = 0; c < 2; ++c) {
                        const double t = (double)tH[c][k] + (double)tL[c][k];
                        o[c] = (t - rd[c == 0 ? RD_CX : RD_CY]) + t * ep -
                               ((double)dh[c][k] + (double)dl[c][k]) * itz;
                    }
                    double ax, ay;
                    const double u = (o[0] * o[0] + o[1] * o[1]) * (rd[6] * rd[6]);
                    if (code == LENSGB_LENS_TNFW && u >= rd[10]) {
                        // a strong TNFW halo outside x = max(tau, 1): the record's
                        // polynomial of the bracket (within 1.3e-9 relative)
                        const double e = rsqrt(u), t = fma(rd[12], e, -1.0);
                        double bs = rd[14 + TNFW_NC - 1];
                        for (int q = TNFW_NC - 2; q >= 0; --q) bs = fma(bs, t, rd[14 + q]);
                        const double a = rd[11] * bs * (e * e);
                        ax = a * o[0];
                        ay = a * o[1];
                    } else {
                        lens_deflect<double>(code, rd, cd, o[0], o[1], ax, ay);
                    }
                    float h, l;
                    split_double(ax, h, l);
                    pair_add(ph[0][k], pq[0][k], h, l);
                    split_double(ay, h, l);
                    pair_add(ph[1][k], pq[1][k], h, l);
                }
            } else {
                float ox[MP_RPT], oy[MP_RPT];
                offsets(rf, ox, oy);
                // the profile switch outside the ray loop, so that the rays'
                // evaluations interleave
                if (code == LENSGB_LENS_TNFW) {
                    tnfw_rays(rf, ox, oy);
                } else {
                    const float* cf = coef_f ? coef_f + g * EPL_NMAX : nullptr;
#pragma unroll
                    for (int k = 0; k < MP_RPT; ++k) {
                        float ax, ay;
                        lens_deflect<float>(code, rf, cf, ox[k], oy[k], ax, ay);
                        s32[0][k] += ax;
                        s32[1][k] += ay;
                    }
                }
            }
        }
        // this chunk's buffer is overwritten by the copy issued next iteration
        __syncthreads();
    }
    const int last = n_steps - 1;
    const double tz = Tz[last];
#pragma unroll
    for (int k = 0; k < MP_RPT; ++k) {
        const long long i = i0 + (long long)k * MP_THREADS;
        if (i >= n) continue;
        double b[2];
        if (!F32) {
            b[0] = xs[0][k] / tz;
            b[1] = xs[1][k] / tz;
        } else {
            const double ep = eps_d[last];
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                // the last plane's deflections move no later position: beta
                // needs d only
                const double t = (double)tH[c][k] + (double)tL[c][k];
                b[c] = t + t * ep - ((double)dh[c][k] + (double)dl[c][k]) / tz;
            }
        }
        bx[i] = b[0];
        by[i] = b[1];
    }
}

// FP64 multi-plane: 1 / T_z per step (into the eps_d scratch, unused in FP64).
__global__ void inv_tz_kernel(const double* __restrict__ Tz, int n, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = 1.0 / Tz[i];
}

int launch_multi_plane(int* tag, const double* rec_d, const float* rec_f, const double* coef_d,
                       const float* coef_f, float* pl_f, double* eps_d, const double* dT,
                       const double* Tz, const double* r2p, int n_steps, const double* ax,
                       const double* ay, double* bx, double* by, long long n, int precision,
                       cudaStream_t stream) {
    if (n <= 0 || n_steps <= 0) return 0;
    const bool f32 = precision == LENSGB_FP32_SPLIT;
    if (f32)
        plane_prepare_kernel<<<(n_steps + PREP_THREADS - 1) / PREP_THREADS, PREP_THREADS, 0,
                               stream>>>(dT, Tz, r2p, n_steps, tag, pl_f, eps_d);
    const long long per_cta = (long long)MP_THREADS * MP_RPT;
    const long long blocks = (n + per_cta - 1) / per_cta;
    if (f32)
        multi_plane_kernel<true><<<(unsigned)blocks, MP_THREADS, 0, stream>>>(
            tag, rec_d, rec_f, coef_d, coef_f, pl_f, eps_d, dT, Tz, r2p, n_steps, ax, ay, bx, by,
            n);
    else {
        inv_tz_kernel<<<(n_steps + 255) / 256, 256, 0, stream>>>(Tz, n_steps, eps_d);
        multi_plane_kernel<false><<<(unsigned)blocks, MP_THREADS, 0, stream>>>(
            tag, rec_d, rec_f, coef_d, coef_f, pl_f, eps_d, dT, Tz, r2p, n_steps, ax, ay, bx, by,
            n);
    }
    return 0;
}

int launch_bulk_ray_shooting(const int* tag, const double* rec_d, const float* rec_f,
                             const double* coef_d, const float* coef_f, int n_defl,
                             const double* x, const double* y, double* bx, double* by,
                             long long n, int precision, cudaStream_t stream) {
    if (n <= 0) return 0;
    const long long per_cta = (long long)BULK_THREADS * BULK_RPT;
    const long long blocks = (n + per_cta - 1) / per_cta;
    if (precision == LENSGB_FP32_SPLIT)
        bulk_ray_kernel<true><<<(unsigned)blocks, BULK_THREADS, 0, stream>>>(
            tag, rec_d, rec_f, coef_d, coef_f, n_defl, x, y, bx, by, n);
    else
        bulk_ray_kernel<false><<<(unsigned)blocks, BULK_THREADS, 0, stream>>>(
            tag, rec_d, rec_f, coef_d, coef_f, n_defl, x, y, bx, by, n);
    return 0;
}

}  // namespace lensgb
