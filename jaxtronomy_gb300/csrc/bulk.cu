// Many-deflector ray shooting: SinglePlaneBulk.ray_shooting
// (JAXtronomy LensModel/single_plane_bulk.py:109-131), beta = x - sum_i alpha_i.
//
// The reference materialises an [n_deflectors, n_rays] FP64 array through
// lax.map + lax.switch and sums it.  Here one thread owns one ray and walks
// the deflector list; the block stages the FP32 records and tags of 64
// deflectors at a time in shared memory, so every thread of a warp evaluates
// the same deflector (the profile switch is warp-uniform).  In FP32_SPLIT
// mode a deflector tagged FP32 is evaluated from the split centre
// (x_hi - c_hi) + (x_lo - c_lo) and summed in FP32 within the chunk; chunk
// sums and FP64-tagged terms accumulate in FP64.
#include "launch.h"
#include "profiles.cuh"

namespace lensgb {

constexpr int BULK_CHUNK = 64;
constexpr int BULK_THREADS = 256;

template <bool F32>
__global__ void __launch_bounds__(BULK_THREADS)
bulk_ray_kernel(const int* __restrict__ tag, const double* __restrict__ rec_d,
                const float* __restrict__ rec_f, const double* __restrict__ coef_d,
                const float* __restrict__ coef_f, int n_defl, const double* __restrict__ x,
                const double* __restrict__ y, double* __restrict__ bx, double* __restrict__ by,
                long long n) {
    __shared__ __align__(16) float srec[BULK_CHUNK * REC_F];
    __shared__ int stag[BULK_CHUNK];
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < n;
    const double xd = live ? x[i] : 0.0;
    const double yd = live ? y[i] : 0.0;
    float xh, xl, yh, yl;
    split_double(xd, xh, xl);
    split_double(yd, yh, yl);
    double axd = 0.0, ayd = 0.0;
    for (int c0 = 0; c0 < n_defl; c0 += BULK_CHUNK) {
        const int cnt = n_defl - c0 < BULK_CHUNK ? n_defl - c0 : BULK_CHUNK;
        __syncthreads();
        if (F32) {
            const float* src = rec_f + (long long)c0 * REC_F;
            for (int k = threadIdx.x; k < cnt * REC_F; k += blockDim.x) srec[k] = src[k];
        }
        for (int k = threadIdx.x; k < cnt; k += blockDim.x) stag[k] = tag[c0 + k];
        __syncthreads();
        float sx = 0.f, sy = 0.f;
        for (int j = 0; j < cnt; ++j) {
            const int t = stag[j];
            const int code = t & BULK_CODE_MASK;
            if (code == LENSGB_LENS_NULL) continue;
            const long long g = c0 + j;
            if (!F32 || (t & BULK_TAG_FP64)) {
                const double* rd = rec_d + g * REC_D;
                const double* cd = coef_d ? coef_d + g * EPL_NMAX : nullptr;
                double ax, ay;
                lens_deflect<double>(code, rd, cd, xd - rd[RD_CX], yd - rd[RD_CY], ax, ay);
                axd += ax;
                ayd += ay;
            } else {
                const float* rf = srec + j * REC_F;
                const float* cf = coef_f ? coef_f + g * EPL_NMAX : nullptr;
                const float dx = __fadd_rn(__fsub_rn(xh, rf[RF_X0H]), __fsub_rn(xl, rf[RF_X0L]));
                const float dy = __fadd_rn(__fsub_rn(yh, rf[RF_Y0H]), __fsub_rn(yl, rf[RF_Y0L]));
                float ax, ay;
                lens_deflect<float>(code, rf, cf, dx, dy, ax, ay);
                sx += ax;
                sy += ay;
            }
        }
        axd += (double)sx;
        ayd += (double)sy;
    }
    if (live) {
        bx[i] = xd - axd;
        by[i] = yd - ayd;
    }
}

int launch_bulk_ray_shooting(const int* tag, const double* rec_d, const float* rec_f,
                             const double* coef_d, const float* coef_f, int n_defl,
                             const double* x, const double* y, double* bx, double* by,
                             long long n, int precision, cudaStream_t stream) {
    if (n <= 0) return 0;
    const long long blocks = (n + BULK_THREADS - 1) / BULK_THREADS;
    if (precision == LENSGB_FP32_SPLIT)
        bulk_ray_kernel<true><<<(unsigned)blocks, BULK_THREADS, 0, stream>>>(
            tag, rec_d, rec_f, coef_d, coef_f, n_defl, x, y, bx, by, n);
    else
        bulk_ray_kernel<false><<<(unsigned)blocks, BULK_THREADS, 0, stream>>>(
            tag, rec_d, rec_f, coef_d, coef_f, n_defl, x, y, bx, by, n);
    return 0;
}

}  // namespace lensgb
