// Image log-likelihood reduction (one CTA per system, FP64 accumulation with
// Kahan-compensated per-thread partial sums and a fixed-order tree combine, so
// results are bit-identical run to run).
//
//   logL = -1/2 sum_pix mask * (m - d)^2 / (C_D(m) + |err|)
//   C_D(m) = noise_map^2                            if a noise map is given
//          = max(m, 0) / exposure + background_rms^2  otherwise
//
// Reference: JAXtronomy Data/imaging_data.py:159-182 (ImageData._log_likelihood),
// Data/image_noise.py:100-137 (C_D_model, covariance_matrix), exposure floor
// image_noise.py:52-54 (applied by the host when the exposure map is built).
#include "launch.h"

namespace lensgb {

constexpr int LL_THREADS = 256;

template <typename R>
__global__ void __launch_bounds__(LL_THREADS)
loglike_kernel(const R* __restrict__ model, long long npix, LoglikeArgs a,
               double* __restrict__ out) {
    const int inst = blockIdx.x;
    const R* m = model + (long long)inst * npix;
    const double* d = a.data + (long long)inst * a.data_stride;
    const double* nm = a.noise_map ? a.noise_map + (long long)inst * a.noise_stride : nullptr;
    const double* ex = a.exposure ? a.exposure + (long long)inst * a.exposure_stride : nullptr;
    const double* mask = a.mask ? a.mask + (long long)inst * a.mask_stride : nullptr;
    const double b2 = a.background_rms * a.background_rms;
    double sum = 0.0, comp = 0.0;
    for (long long i = threadIdx.x; i < npix; i += LL_THREADS) {
        const double mk = mask ? mask[i] : 1.0;
        if (mk == 0.0) continue;
        const double mv = (double)m[i];
        double c;
        if (nm) {
            c = nm[i] * nm[i];
        } else {
            const double e = ex ? ex[i] : a.exposure_time;
            c = (mv >= 0 ? mv : 0.0) / e + b2;
        }
        if (a.error_map) c += fabs(a.error_map[i]);
        const double r = mv - d[i];
        const double term = r * r / c * mk;
        // Kahan summation
        const double y = term - comp;
        const double t = sum + y;
        comp = (t - sum) - y;
        sum = t;
    }
    __shared__ double red[LL_THREADS];
    red[threadIdx.x] = sum;
    __syncthreads();
    for (int w = LL_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[inst] = -red[0] / 2.0;
}

int launch_loglike(const void* model, int n_inst, long long npix, const LoglikeArgs& a,
                   double* out, int precision, cudaStream_t stream) {
    if (n_inst <= 0) return 0;
    if (precision == LENSGB_FP64)
        loglike_kernel<double><<<n_inst, LL_THREADS, 0, stream>>>((const double*)model, npix, a,
                                                                  out);
    else
        loglike_kernel<float><<<n_inst, LL_THREADS, 0, stream>>>((const float*)model, npix, a,
                                                                 out);
    return 0;
}

}  // namespace lensgb
