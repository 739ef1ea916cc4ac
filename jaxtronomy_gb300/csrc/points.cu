// Point-wise FP64 kernels behind LensModel.ray_shooting and
// LightModel.surface_brightness for arbitrary coordinate arrays and one
// parameter set (JAXtronomy LensModel/single_plane.py:39-56,113-139 and
// LightModel/light_model_base.py:230-252).  One thread per point.
#include "launch.h"
#include "profiles.cuh"

namespace lensgb {

__global__ void ray_shoot_points_kernel(StackDesc st, const double* __restrict__ rec,
                                        const double* __restrict__ coef,
                                        const double* __restrict__ x, const double* __restrict__ y,
                                        double* __restrict__ bx, double* __restrict__ by,
                                        long long n, int want_alpha) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double X = x[i], Y = y[i];
    double axs = 0, ays = 0;
    for (int p = 0; p < st.n_lens; ++p) {
        const double* r = rec + p * REC_D;
        const int es = st.epl_slot[p];
        double ax, ay;
        lens_deflect<double>(st.lens[p], r, es >= 0 ? coef + es * EPL_NMAX : nullptr, X - r[RD_CX],
                       Y - r[RD_CY], ax, ay);
        axs += ax;
        ays += ay;
    }
    if (want_alpha) {
        bx[i] = axs * st.alpha_scaling;
        by[i] = ays * st.alpha_scaling;
    } else {
        bx[i] = X - axs * st.alpha_scaling;
        by[i] = Y - ays * st.alpha_scaling;
    }
}

__global__ void light_points_kernel(StackDesc st, int which, const double* __restrict__ rec,
                                    const double* __restrict__ x, const double* __restrict__ y,
                                    double* __restrict__ out, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double X = x[i], Y = y[i];
    const int base = st.n_lens + (which == 0 ? 0 : st.n_src);
    const int cnt = which == 0 ? st.n_src : st.n_ll;
    double f = 0;
    for (int k = 0; k < cnt; ++k) {
        const double* r = rec + (base + k) * REC_D;
        f += sersic_flux<double>(r, X - r[RD_CX], Y - r[RD_CY]);
    }
    out[i] = f;
}

int launch_ray_shoot_points(const StackDesc& st, const double* rec_d, const double* coef_d,
                            const double* x, const double* y, double* bx, double* by,
                            long long n, int want_alpha, cudaStream_t stream) {
    if (n <= 0) return 0;
    int threads = 256;
    long long blocks = (n + threads - 1) / threads;
    ray_shoot_points_kernel<<<(unsigned)blocks, threads, 0, stream>>>(st, rec_d, coef_d, x, y, bx,
                                                                        by, n, want_alpha);
    return 0;
}

int launch_light_points(const StackDesc& st, int which, const double* rec_d, const double* x,
                        const double* y, double* out, long long n, cudaStream_t stream) {
    if (n <= 0) return 0;
    int threads = 256;
    long long blocks = (n + threads - 1) / threads;
    light_points_kernel<<<(unsigned)blocks, threads, 0, stream>>>(st, which, rec_d, x, y, out, n);
    return 0;
}

}  // namespace lensgb
