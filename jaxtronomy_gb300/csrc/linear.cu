// Linear amplitude solve of ImageLinearFit (JAXtronomy ImSim/image_linear_solve.py:98-228,
// 229-341) for a batch of systems: one CTA per system.
//
//   A_j      unit-amplitude convolved image of linear component j (the caller's
//            lensgb_image of component j alone with amp = 1; :362-456)
//   W        mask / C_D(data): noise_map^2, or max(d, 0) / exposure + bkg^2
//            (the data-based covariance of error_response; image_noise.py:115-137)
//   M = A W A^T, R = A W d, solved when cond(M) < 5 / eps, else zero amplitudes
//            (de_lens.get_param_WLS, de_lens.py:8-38)
//   model    sum_j B_j A_j on the mask, 0 elsewhere (array_masked2image)
//   logL     ImageData.log_likelihood(model, mask) with the model-based C_D
//            (imaging_data.py:159-182), + 1/2 log det(M^-1) with source_marg
//            (marginalisation_const, de_lens.py:41-49), - 1e8 if check_positive_flux
//            finds a negative amplitude (image_linear_solve.py:320-340, 598-618)
//
// FP64 throughout; reductions are warp shuffles in a fixed order, so results are
// bit-identical run to run.
#include <math.h>

#include "launch.h"

namespace lensgb {

constexpr int LIN_THREADS = 256;
constexpr int LIN_WARPS = LIN_THREADS / 32;
constexpr int LIN_NACC = LIN_MAX * (LIN_MAX + 1) / 2 + LIN_MAX;  // upper triangle of M, then R

// Warp sum in a fixed order (lane 0 holds the result).
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Eigenvalues of a symmetric n x n matrix (cyclic Jacobi; n <= LIN_MAX).
__device__ void sym_eigenvalues(double (*a)[LIN_MAX], int n, double* ev) {
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0.0;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) off += a[p][q] * a[p][q];
        if (off == 0.0) break;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                if (a[p][q] == 0.0) continue;
                const double th = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
                const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {
                    const double akp = a[k][p], akq = a[k][q];
                    a[k][p] = c * akp - s * akq;
                    a[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    const double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = c * apk - s * aqk;
                    a[q][k] = s * apk + c * aqk;
                }
            }
    }
    for (int i = 0; i < n; ++i) ev[i] = a[i][i];
}

// Solves M X = B for `nb` right-hand sides (columns of b) by Gaussian elimination
// with partial pivoting; returns the sign of det(M) (0: singular) and log|det|.
__device__ int lu_solve(double (*m)[LIN_MAX], int n, double (*b)[LIN_MAX], int nb,
                        double* logabsdet) {
    int sign = 1;
    double ld = 0.0;
    for (int c = 0; c < n; ++c) {
        int piv = c;
        for (int r = c + 1; r < n; ++r)
            if (fabs(m[r][c]) > fabs(m[piv][c])) piv = r;
        if (m[piv][c] == 0.0) {
            *logabsdet = -INFINITY;
            return 0;
        }
        if (piv != c) {
            sign = -sign;
            for (int k = 0; k < n; ++k) {
                const double t = m[c][k];
                m[c][k] = m[piv][k];
                m[piv][k] = t;
            }
            for (int k = 0; k < nb; ++k) {
                const double t = b[c][k];
                b[c][k] = b[piv][k];
                b[piv][k] = t;
            }
        }
        const double d = m[c][c];
        if (d < 0) sign = -sign;
        ld += log(fabs(d));
        for (int r = c + 1; r < n; ++r) {
            const double f = m[r][c] / d;
            if (f == 0.0) continue;
            for (int k = c; k < n; ++k) m[r][k] -= f * m[c][k];
            for (int k = 0; k < nb; ++k) b[r][k] -= f * b[c][k];
        }
    }
    for (int k = 0; k < nb; ++k)
        for (int r = n - 1; r >= 0; --r) {
            double v = b[r][k];
            for (int c = r + 1; c < n; ++c) v -= m[r][c] * b[c][k];
            b[r][k] = v / m[r][r];
        }
    *logabsdet = ld;
    return sign;
}

template <typename R>
__global__ void __launch_bounds__(LIN_THREADS)
linear_solve_kernel(const R* __restrict__ A, int n_lin, int n_inst, long long npix,
                    LoglikeArgs a, int flags, double* __restrict__ param,
                    double* __restrict__ cov, R* __restrict__ image, double* __restrict__ logl) {
    const int inst = blockIdx.x;
    const int n = n_lin;
    const double* d = a.data + (long long)inst * a.data_stride;
    const double* nm = a.noise_map ? a.noise_map + (long long)inst * a.noise_stride : nullptr;
    const double* ex = a.exposure ? a.exposure + (long long)inst * a.exposure_stride : nullptr;
    const double* mask = a.mask ? a.mask + (long long)inst * a.mask_stride : nullptr;
    const double b2 = a.background_rms * a.background_rms;
    const long long cstride = (long long)n_inst * npix;  // between components
    const R* Ai = A + (long long)inst * npix;

    // pass 1: M (upper triangle) and R over the mask, weighted by 1 / C_D(data)
    double acc[LIN_NACC];
#pragma unroll
    for (int k = 0; k < LIN_NACC; ++k) acc[k] = 0.0;
    for (long long p = threadIdx.x; p < npix; p += LIN_THREADS) {
        const double mk = mask ? mask[p] : 1.0;
        if (mk == 0.0) continue;
        const double dv = d[p];
        double c;
        if (nm) {
            c = nm[p] * nm[p];
        } else {
            const double e = ex ? ex[p] : a.exposure_time;
            c = (dv >= 0 ? dv : 0.0) / e + b2;
        }
        const double w = 1.0 / c;
        double av[LIN_MAX];
#pragma unroll
        for (int j = 0; j < LIN_MAX; ++j) av[j] = j < n ? (double)Ai[j * cstride + p] : 0.0;
        int k = 0;
#pragma unroll
        for (int j = 0; j < LIN_MAX; ++j)
#pragma unroll
            for (int l = j; l < LIN_MAX; ++l) acc[k++] += av[j] * w * av[l];
#pragma unroll
        for (int j = 0; j < LIN_MAX; ++j) acc[k++] += av[j] * w * dv;
    }
    __shared__ double part[LIN_WARPS][LIN_NACC];
    __shared__ double sol[LIN_MAX];
    __shared__ double corr;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < LIN_NACC; ++k) {
        const double v = warp_sum(acc[k]);
        if (lane == 0) part[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double Mt[LIN_MAX][LIN_MAX], Rv[LIN_MAX];
        int k = 0;
        for (int j = 0; j < LIN_MAX; ++j)
            for (int l = j; l < LIN_MAX; ++l, ++k) {
                double v = 0.0;
                for (int w = 0; w < LIN_WARPS; ++w) v += part[w][k];
                if (j < n && l < n) Mt[j][l] = Mt[l][j] = v;
            }
        for (int j = 0; j < LIN_MAX; ++j, ++k) {
            double v = 0.0;
            for (int w = 0; w < LIN_WARPS; ++w) v += part[w][k];
            if (j < n) Rv[j] = v;
        }
        // stability: 2-norm condition number of the symmetric M below 5 / eps
        double e[LIN_MAX][LIN_MAX], ev[LIN_MAX];
        for (int j = 0; j < n; ++j)
            for (int l = 0; l < n; ++l) e[j][l] = Mt[j][l];
        sym_eigenvalues(e, n, ev);
        double lmax = 0.0, lmin = INFINITY;
        for (int j = 0; j < n; ++j) {
            lmax = fmax(lmax, fabs(ev[j]));
            lmin = fmin(lmin, fabs(ev[j]));
        }
        const bool stable = lmin > 0.0 && lmax / lmin < 5.0 / 2.220446049250313e-16;
        double x[LIN_MAX];
        double marg = 0.0;
        if (flags & LENSGB_LINEAR_INVERSE) {
            // M^-1 (zeros if M is not invertible), then B = M^-1 R
            double lu[LIN_MAX][LIN_MAX], inv[LIN_MAX][LIN_MAX];
            for (int j = 0; j < n; ++j)
                for (int l = 0; l < n; ++l) {
                    lu[j][l] = Mt[j][l];
                    inv[j][l] = j == l ? 1.0 : 0.0;
                }
            double ld;
            const int sg = lu_solve(lu, n, inv, n, &ld);
            for (int j = 0; j < n; ++j)
                for (int l = 0; l < n; ++l) {
                    double v = (stable && sg != 0) ? inv[j][l] : 0.0;
                    if (!isfinite(v)) v = 0.0;
                    inv[j][l] = v;
                }
            for (int j = 0; j < n; ++j) {
                double v = 0.0;
                for (int l = 0; l < n; ++l) v += inv[j][l] * Rv[l];
                x[j] = v;
            }
            if (cov)
                for (int j = 0; j < n; ++j)
                    for (int l = 0; l < n; ++l)
                        cov[((long long)inst * n + j) * n + l] = inv[j][l];
            // marginalisation constant: sign * log|det(M^-1)| / 2, -1e15 if singular
            double lu2[LIN_MAX][LIN_MAX], dummy[LIN_MAX][LIN_MAX];
            for (int j = 0; j < n; ++j)
                for (int l = 0; l < n; ++l) lu2[j][l] = inv[j][l];
            double ld2;
            const int sg2 = lu_solve(lu2, n, dummy, 0, &ld2);
            marg = sg2 == 0 ? -1e15 : sg2 * ld2 / 2.0;
        } else {
            double lu[LIN_MAX][LIN_MAX], rhs[LIN_MAX][LIN_MAX];
            for (int j = 0; j < n; ++j) {
                for (int l = 0; l < n; ++l) lu[j][l] = Mt[j][l];
                rhs[j][0] = Rv[j];
            }
            double ld;
            const int sg = lu_solve(lu, n, rhs, 1, &ld);
            bool finite = sg != 0;
            for (int j = 0; j < n; ++j) finite = finite && isfinite(rhs[j][0]);
            for (int j = 0; j < n; ++j) x[j] = (stable && finite) ? rhs[j][0] : 0.0;
        }
        bool negative = false;
        for (int j = 0; j < n; ++j) {
            sol[j] = x[j];
            param[(long long)inst * n + j] = x[j];
            negative = negative || x[j] < 0.0;
        }
        corr = marg - ((flags & LENSGB_LINEAR_POSITIVE) && negative ? 1e8 : 0.0);
    }
    __syncthreads();

    // pass 2: the model image and its log-likelihood (model-based C_D)
    double B[LIN_MAX];
#pragma unroll
    for (int j = 0; j < LIN_MAX; ++j) B[j] = j < n ? sol[j] : 0.0;
    R* img = image + (long long)inst * npix;
    double sum = 0.0, comp = 0.0;
    for (long long p = threadIdx.x; p < npix; p += LIN_THREADS) {
        const double mk = mask ? mask[p] : 1.0;
        double mv = 0.0;
        if (mk != 0.0) {
#pragma unroll
            for (int j = 0; j < LIN_MAX; ++j)
                if (j < n) mv += (double)Ai[j * cstride + p] * B[j];
        }
        img[p] = (R)mv;
        if (mk == 0.0) continue;
        double c;
        if (nm) {
            c = nm[p] * nm[p];
        } else {
            const double e = ex ? ex[p] : a.exposure_time;
            c = (mv >= 0 ? mv : 0.0) / e + b2;
        }
        if (a.error_map) c += fabs(a.error_map[p]);
        const double r = mv - d[p];
        const double term = r * r / c * mk;
        const double y = term - comp;
        const double t = sum + y;
        comp = (t - sum) - y;
        sum = t;
    }
    __shared__ double red[LIN_WARPS];
    const double ws = warp_sum(sum);
    if (lane == 0) red[warp] = ws;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < LIN_WARPS; ++w) s += red[w];
        logl[inst] = -s / 2.0 + corr;
    }
}

int launch_linear_solve(const void* A, int n_lin, int n_inst, long long npix, const LoglikeArgs& a,
                        int flags, double* param, double* cov, void* image, double* logl,
                        int precision, cudaStream_t stream) {
    if (n_inst <= 0) return 0;
    if (precision == LENSGB_FP64)
        linear_solve_kernel<double><<<n_inst, LIN_THREADS, 0, stream>>>(
            (const double*)A, n_lin, n_inst, npix, a, flags, param, cov, (double*)image, logl);
    else
        linear_solve_kernel<float><<<n_inst, LIN_THREADS, 0, stream>>>(
            (const float*)A, n_lin, n_inst, npix, a, flags, param, cov, (float*)image, logl);
    return 0;
}

}  // namespace lensgb
