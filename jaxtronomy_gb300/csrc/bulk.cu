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

constexpr int BULK_CHUNK = 64;
constexpr int BULK_THREADS = 256;
constexpr int BULK_RPT = 2;  // rays per thread (i and i + BULK_THREADS of the CTA span)

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
    double xd[BULK_RPT], yd[BULK_RPT], axd[BULK_RPT], ayd[BULK_RPT];
    float xh[BULK_RPT], xl[BULK_RPT], yh[BULK_RPT], yl[BULK_RPT];
#pragma unroll
    for (int k = 0; k < BULK_RPT; ++k) {
        const long long i = i0 + (long long)k * BULK_THREADS;
        xd[k] = i < n ? x[i] : 0.0;
        yd[k] = i < n ? y[i] : 0.0;
        split_double(xd[k], xh[k], xl[k]);
        split_double(yd[k], yh[k], yl[k]);
        axd[k] = 0.0;
        ayd[k] = 0.0;
    }
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
            const int code = t & BULK_CODE_MASK;
            if (code == LENSGB_LENS_NULL) continue;
            const long long g = c0 + j;
            if (!F32 || (t & BULK_TAG_FP64)) {
                const double* rd = rec_d + g * REC_D;
                const double* cd = coef_d ? coef_d + g * EPL_NMAX : nullptr;
#pragma unroll
                for (int k = 0; k < BULK_RPT; ++k) {
                    double ax, ay;
                    lens_deflect<double>(code, rd, cd, xd[k] - rd[RD_CX], yd[k] - rd[RD_CY], ax,
                                         ay);
                    axd[k] += ax;
                    ayd[k] += ay;
                }
            } else {
                const float* rf = srec + j * REC_F;
                const float ch = rf[RF_X0H], cl = rf[RF_X0L], dh = rf[RF_Y0H], dl = rf[RF_Y0L];
                if (code == LENSGB_LENS_TNFW) {
                    // the subhalo case: fused FP32 pair evaluation
#pragma unroll
                    for (int k = 0; k < BULK_RPT; ++k) {
                        const float dx = __fadd_rn(__fsub_rn(xh[k], ch), __fsub_rn(xl[k], cl));
                        const float dy = __fadd_rn(__fsub_rn(yh[k], dh), __fsub_rn(yl[k], dl));
                        float ax, ay;
                        tnfw_pair_f(rf, dx, dy, ax, ay);
                        sx[k] += ax;
                        sy[k] += ay;
                    }
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
            bx[i] = xd[k] - axd[k];
            by[i] = yd[k] - ayd[k];
        }
    }
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
