// Point-source rendering: PointSourceRendering.point_source_rendering
// (JAXtronomy ImSim/Numerics/point_source_rendering.py:34-77) as used by
// ImageModel.point_source (ImSim/image_model.py:396-429).
//
// The reference paints, for every image i at pixel position (x_i, y_i) =
// Ma2pix (ra, dec) + (x0, y0), the kernel K (k x k, at subgrid factor p)
// bilinearly interpolated (jax.scipy.ndimage.map_coordinates, order 1, zero
// outside K; Util/image_util.py:9-40) at kernel coordinates
//   (row, col) = (i_s + k/2 - y_s, j_s + k/2 - x_s),  x_s = p x_i + (p - 1)/2,
// onto a p-times finer grid, then averages p x p blocks and multiplies by p^2
// (image_util.re_size), i.e. sums the p x p cells of each pixel.
//
// Here one thread owns one output pixel and gathers over the images of its
// system (deterministic, no atomics).  Within a pixel the p x p cells share
// one fractional offset, so the p^2 bilinear samples collapse into a weighted
// sum over the (p + 1) x (p + 1) kernel window starting at floor(row), floor(col):
// edge rows / columns weighted by (1 - f) and f, interior ones by 1.
#include "launch.h"

namespace lensgb {

constexpr int PS_THREADS = 256;

template <typename R>
__global__ void __launch_bounds__(PS_THREADS)
point_source_kernel(const double* __restrict__ ps, int n_img, const double* __restrict__ K,
                    int ks, long long kstride, int p, double m00, double m01, double m10,
                    double m11, double x0, double y0, int nx, int ny, double scale,
                    R* __restrict__ out) {
    const int b = blockIdx.y;
    const long long pix = (long long)blockIdx.x * PS_THREADS + threadIdx.x;
    if (pix >= (long long)nx * ny) return;
    const int r = (int)(pix / ny), c = (int)(pix % ny);
    const double* kb = K + (long long)b * kstride;
    const int h = ks / 2;
    R acc = R(0);
    for (int i = 0; i < n_img; ++i) {
        const double* q = ps + ((long long)b * n_img + i) * 3;
        const double ra = q[0], dec = q[1], amp = q[2];
        const double xp = m00 * ra + m01 * dec + x0;
        const double yp = m10 * ra + m11 * dec + y0;
        const double xs = xp * p + (p - 1) / 2.0;
        const double ys = yp * p + (p - 1) / 2.0;
        // kernel coordinates of this pixel's first cell
        const double u0 = (double)r * p + h - ys, v0 = (double)c * p + h - xs;
        if (!(u0 > -(double)p - 1.0 && u0 < (double)ks && v0 > -(double)p - 1.0 &&
              v0 < (double)ks))
            continue;  // the pixel's cells miss the kernel (also skips NaN positions)
        const double fu_ = floor(u0), fv_ = floor(v0);
        const int iu = (int)fu_, iv = (int)fv_;
        const R fu = (R)(u0 - fu_), fv = (R)(v0 - fv_);
        R s = R(0);
        for (int m = 0; m <= p; ++m) {
            const int row = iu + m;
            if (row < 0 || row >= ks) continue;
            const R wr = m == 0 ? R(1) - fu : (m == p ? fu : R(1));
            R sr = R(0);
            for (int n = 0; n <= p; ++n) {
                const int col = iv + n;
                if (col < 0 || col >= ks) continue;
                const R wc = n == 0 ? R(1) - fv : (n == p ? fv : R(1));
                sr += wc * (R)kb[(long long)row * ks + col];
            }
            s += wr * sr;
        }
        acc += (R)amp * s;
    }
    if (acc != R(0)) out[(long long)b * nx * ny + pix] += acc * (R)scale;
}

int launch_point_sources(const double* ps, int n_img, int n_inst, const double* K, int ks,
                         long long kstride, int p, const double* Ma2pix, double x0, double y0,
                         int nx, int ny, double scale, void* out, int precision,
                         cudaStream_t stream) {
    if (n_inst <= 0 || n_img <= 0) return 0;
    const long long npix = (long long)nx * ny;
    dim3 grid((unsigned)((npix + PS_THREADS - 1) / PS_THREADS), (unsigned)n_inst);
    if (precision == LENSGB_FP64)
        point_source_kernel<double><<<grid, PS_THREADS, 0, stream>>>(
            ps, n_img, K, ks, kstride, p, Ma2pix[0], Ma2pix[1], Ma2pix[2], Ma2pix[3], x0, y0, nx,
            ny, scale, (double*)out);
    else
        point_source_kernel<float><<<grid, PS_THREADS, 0, stream>>>(
            ps, n_img, K, ks, kstride, p, Ma2pix[0], Ma2pix[1], Ma2pix[2], Ma2pix[3], x0, y0, nx,
            ny, scale, (float*)out);
    return 0;
}

}  // namespace lensgb
