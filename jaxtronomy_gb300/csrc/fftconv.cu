// "same"-mode 2-D convolution by FP64 FFT in shared memory, for large kernels
// (zero padding, or edge padding through an explicitly padded image).
//
// The reference convolves with jax.scipy.signal.fftconvolve(image, kernel,
// mode="same") (JAXtronomy ImSim/Numerics/convolution.py:80-81): the full
// linear convolution, cropped to the image's size and centre (rows and columns
// h .. h + N - 1 for an odd K = 2h + 1).  Here, per system, with P the power of
// two >= N + K - 1 (so the circular convolution of the zero-padded arrays has
// no wrap-around):
//   1. fft_rows_fwd_kernel: the N image rows, zero-padded to P, are
//      transformed (one CTA per group of rows; radix-2 in shared memory);
//   2. fft_cols_kernel: each CTA takes a group of columns of that N x P array
//      (rows >= N are zero), transforms them, multiplies by the kernel's
//      spectrum, transforms back and keeps only rows h .. h + N - 1 -- the
//      whole column pass of the 2-D transform and the product stay in shared
//      memory;
//   3. fft_rows_inv_kernel: those N rows are transformed back and columns
//      h .. h + N - 1, divided by P^2, are the output.
// The kernel's spectrum (its zero-padded P x P transform) comes from the same
// two passes without the product (fft_cols_kernel with mul = null), once per
// distinct kernel.  Edge padding (GaussianConvolution, convolution.py:215-235)
// transforms the (N + 2h)-square edge-padded image instead and keeps the
// outputs h further in.  Everything is FP64: an FP32 transform's rounding
// (~1e-7 of the image maximum) would be a 1e-4 relative error on pixels at
// 1e-3 of the maximum.  Twiddles e^{-2 pi i k / P} come from sincospi in FP64.
//
// Cost per system ~ 3 x 5 P^2 log2(P) flop (in FP64, whatever the kernel size),
// against 2 K^2 N^2 for the direct kernels: at N = 1200, K = 165 (a 41-pixel
// PSF convolved on a 4x supersampled grid) 0.9 GFLOP against 65 GFLOP.
#include <map>
#include <mutex>

#include "launch.h"

namespace lensgb {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ int bitrev(int v, int lg) {
    return (int)(__brev((unsigned)v) >> (32 - lg));
}

// In-place radix-2 decimation-in-time FFT of nl lines of length P = 2^lg
// (lg >= 1) held in shared memory (line l at buf + l * P), loaded in
// bit-reversed order.  inverse: conjugate twiddles (no 1/P).
__device__ void fft_lines(double2* buf, int nl, int P, int lg, const double2* __restrict__ tw,
                          bool inverse) {
    const int half_p = P >> 1;
    const int total = nl * half_p;
    for (int half = 1, step = half_p; half < P; half <<= 1, step >>= 1) {
        for (int t = threadIdx.x; t < total; t += blockDim.x) {
            const int l = t >> (lg - 1), j = t & (half_p - 1);
            const int pos = j & (half - 1);
            const int i0 = ((j - pos) << 1) + pos, i1 = i0 + half;
            double2 w = __ldg(tw + pos * step);
            if (inverse) w.y = -w.y;
            double2* x = buf + (long long)l * P;
            const double2 a = x[i0], b = cmul(x[i1], w);
            x[i0] = make_double2(a.x + b.x, a.y + b.y);
            x[i1] = make_double2(a.x - b.x, a.y - b.y);
        }
        __syncthreads();
    }
}

__global__ void twiddle_kernel(double2* tw, int P) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P / 2) return;
    double s, c;
    sincospi(-2.0 * k / P, &s, &c);
    tw[k] = make_double2(c, s);
}

// Pass 1: rows 0 .. n_rows-1 of each system's real array, zero-padded to P
// columns, transformed; out: (n_sys, n_rows, P).  `rows` rows per CTA,
// blockIdx.y = system.  pad = 0: the array is the (n_rows x n_cols) input.
// pad = h > 0 (edge padding): the array is the (n_rows - 2h) x (n_cols - 2h)
// input grown by h rows and columns on every side that repeat its edge pixels.
template <typename T>
__global__ void __launch_bounds__(256)
fft_rows_fwd_kernel(const T* __restrict__ in, long long in_stride, int n_rows, int n_cols,
                    int pad, double2* __restrict__ out, int P, int lg, int rows,
                    const double2* __restrict__ tw) {
    extern __shared__ double2 sbuf[];
    const int sys = blockIdx.y;
    const int r0 = blockIdx.x * rows;
    const int nl = min(rows, n_rows - r0);
    const T* src = in + sys * in_stride;
    const int sr_max = n_rows - 2 * pad - 1, sc_max = n_cols - 2 * pad - 1;
    const int pitch = n_cols - 2 * pad;
    for (int e = threadIdx.x; e < nl * P; e += blockDim.x) {
        const int l = e / P, c = e - l * P;
        double v = 0.0;
        if (c < n_cols) {
            const int sr = min(max(r0 + l - pad, 0), sr_max), sc = min(max(c - pad, 0), sc_max);
            v = (double)src[(long long)sr * pitch + sc];
        }
        sbuf[l * P + bitrev(c, lg)] = make_double2(v, 0.0);
    }
    __syncthreads();
    fft_lines(sbuf, nl, P, lg, tw, false);
    double2* dst = out + ((long long)sys * n_rows + r0) * P;
    for (int e = threadIdx.x; e < nl * P; e += blockDim.x) dst[e] = sbuf[e];
}

// Pass 2: columns c0 .. c0+cols-1 of each system's (n_rows x P) array (systems
// n_rows x P apart), rows >= n_rows being zero, transformed along the column.
// mul != null: times the spectrum mul (P x P, row-major, mul_stride apart per
// system), transformed back, rows keep0 .. keep0+n_keep-1 written to rows
// 0 .. n_keep-1 of `out` (systems out_stride apart).  mul == null: the full
// transformed columns written to `out` (systems out_stride apart, P x P).
// `in` and `out` may be the same array: a CTA reads all of its columns before
// it writes any of them, no other CTA touches those columns, and out_stride
// equal to the input's system stride keeps the systems apart.
__global__ void __launch_bounds__(256)
fft_cols_kernel(const double2* in, int n_rows, double2* out, long long out_stride, int P, int lg,
                int cols, const double2* __restrict__ mul, long long mul_stride, int keep0,
                int n_keep, const double2* __restrict__ tw) {
    extern __shared__ double2 sbuf[];
    const int sys = blockIdx.y;
    const int c0 = blockIdx.x * cols;
    const double2* src = in + (long long)sys * n_rows * P;
    // line cc = column c0 + cc, element r at bit-reversed position
    for (int e = threadIdx.x; e < cols * P; e += blockDim.x) {
        const int r = e / cols, cc = e - r * cols;
        const double2 v = r < n_rows ? src[(long long)r * P + c0 + cc] : make_double2(0.0, 0.0);
        sbuf[cc * P + bitrev(r, lg)] = v;
    }
    __syncthreads();
    fft_lines(sbuf, cols, P, lg, tw, false);
    double2* dst = out + (long long)sys * out_stride;
    if (!mul) {
        for (int e = threadIdx.x; e < cols * P; e += blockDim.x) {
            const int r = e / cols, cc = e - r * cols;
            dst[(long long)r * P + c0 + cc] = sbuf[cc * P + r];
        }
        return;
    }
    const double2* m = mul + sys * mul_stride;
    // product with the kernel spectrum, re-ordered bit-reversed for the inverse
    // transform into the second half of the buffer
    double2* sb2 = sbuf + cols * P;
    for (int e = threadIdx.x; e < cols * P; e += blockDim.x) {
        const int r = e / cols, cc = e - r * cols;
        sb2[cc * P + bitrev(r, lg)] =
            cmul(sbuf[cc * P + r], __ldg(m + (long long)r * P + c0 + cc));
    }
    __syncthreads();
    fft_lines(sb2, cols, P, lg, tw, true);
    for (int e = threadIdx.x; e < cols * n_keep; e += blockDim.x) {
        const int r = e / cols, cc = e - r * cols;
        dst[(long long)r * P + c0 + cc] = sb2[cc * P + keep0 + r];
    }
}

// Pass 3: rows 0 .. n_rows-1 of each system's array (systems in_stride apart,
// rows P apart) transformed back; columns keep0 .. keep0+n_cols-1 of the real
// part, times scale, are the output rows (n_sys, n_rows, n_cols).
template <typename T>
__global__ void __launch_bounds__(256)
fft_rows_inv_kernel(const double2* __restrict__ in, long long in_stride, int n_rows,
                    T* __restrict__ out, long long out_stride, int n_cols, int P, int lg,
                    int rows, int keep0, double scale, const double2* __restrict__ tw) {
    extern __shared__ double2 sbuf[];
    const int sys = blockIdx.y;
    const int r0 = blockIdx.x * rows;
    const int nl = min(rows, n_rows - r0);
    const double2* src = in + sys * in_stride + (long long)r0 * P;
    for (int e = threadIdx.x; e < nl * P; e += blockDim.x) {
        const int l = e / P, c = e - l * P;
        sbuf[l * P + bitrev(c, lg)] = src[e];
    }
    __syncthreads();
    fft_lines(sbuf, nl, P, lg, tw, true);
    T* dst = out + sys * out_stride + (long long)r0 * n_cols;
    for (int e = threadIdx.x; e < nl * n_cols; e += blockDim.x) {
        const int l = e / n_cols, c = e - l * n_cols;
        dst[(long long)l * n_cols + c] = (T)(sbuf[l * P + keep0 + c].x * scale);
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static int lg2_ceil(long long v) {
    int lg = 0;
    while ((1LL << lg) < v) ++lg;
    return lg;
}

int fft_conv_size(int ny, int nx, int K, int edge) {
    const long long m = (long long)(ny > nx ? ny : nx) + (edge ? K - 1 : 0);
    const long long need = m + K - 1;
    return 1 << lg2_ceil(need < 2 ? 2 : need);
}

size_t fft_conv_scratch_bytes(int n_inst, int ny, int nx, int K, long long kstride, int edge) {
    const long long P = fft_conv_size(ny, nx, K, edge);
    const long long n_k = kstride == 0 ? 1 : n_inst;
    const long long rows = ny + (edge ? K - 1 : 0);
    // twiddles, the row-pass array (rows x P per system, reused by the column
    // pass for its kept rows), the kernel spectra (P x P) and the kernel's row pass
    return (size_t)(P / 2 + (long long)n_inst * rows * P + n_k * P * P + n_k * K * P) * 16 +
           4 * 256;
}

// Lines per CTA: at most 64 KB of shared memory for a row pass (4096 complex
// doubles), 2 x 64 KB for a column pass; a power of two dividing P.
static int rows_per_cta(int P) { return P >= 4096 ? 1 : 4096 / P; }
static int cols_per_cta(int P) {
    const int c = P >= 4096 ? 1 : (4096 / P < 16 ? 4096 / P : 16);
    return c < P ? c : P;
}

static bool set_smem(const void* fn, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, size_t> granted;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(mu);
    size_t& g = granted[std::make_pair(fn, dev)];
    if (bytes <= g) return true;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) !=
        cudaSuccess) {
        cudaGetLastError();  // a refused size leaves no error behind for later calls
        return false;
    }
    g = bytes;
    return true;
}

template <typename T>
static int fft_conv_t(const T* in, T* out, const T* kernel, long long kstride, int n_inst, int ny,
                      int nx, int K, int edge, void* scratch, cudaStream_t stream) {
    const int P = fft_conv_size(ny, nx, K, edge);
    const int lg = lg2_ceil(P);
    if (P > 4096) return -2;
    const int h = K / 2;
    // edge padding: transform the (ny + 2h) x (nx + 2h) edge-padded image and
    // keep the outputs that sit h further in
    const int pad = edge ? h : 0;
    const int my = ny + 2 * pad, mx = nx + 2 * pad, keep0 = h + pad;
    const long long n_k = kstride == 0 ? 1 : n_inst;
    auto align = [](size_t v) { return (v + 255) & ~(size_t)255; };
    unsigned char* base = (unsigned char*)scratch;
    double2* tw = (double2*)base;
    double2* work = (double2*)(base + align((size_t)P / 2 * 16));
    double2* kspec = (double2*)((unsigned char*)work + align((size_t)n_inst * my * P * 16));
    double2* krows = (double2*)((unsigned char*)kspec + align((size_t)n_k * P * P * 16));
    const int rpc = rows_per_cta(P), cpc = cols_per_cta(P);
    const size_t smem_rows = (size_t)rpc * P * 16, smem_cols = (size_t)cpc * P * 16;
    if (!set_smem((const void*)fft_rows_fwd_kernel<T>, smem_rows) ||
        !set_smem((const void*)fft_rows_inv_kernel<T>, smem_rows) ||
        !set_smem((const void*)fft_cols_kernel, 2 * smem_cols))
        return -1;
    twiddle_kernel<<<(P / 2 + 255) / 256, 256, 0, stream>>>(tw, P);
    // kernel spectra: K rows, then full columns
    fft_rows_fwd_kernel<T><<<dim3((K + rpc - 1) / rpc, (unsigned)n_k), 256, smem_rows, stream>>>(
        kernel, kstride, K, K, 0, krows, P, lg, rpc, tw);
    fft_cols_kernel<<<dim3(P / cpc, (unsigned)n_k), 256, smem_cols, stream>>>(
        krows, K, kspec, (long long)P * P, P, lg, cpc, nullptr, 0, 0, 0, tw);
    // image: rows, columns with the product (keeping rows keep0 .. keep0+ny-1,
    // written over the first rows of the same system's array), rows back
    // (keeping columns keep0 .. keep0+nx-1)
    const long long wstride = (long long)my * P;
    fft_rows_fwd_kernel<T><<<dim3((my + rpc - 1) / rpc, (unsigned)n_inst), 256, smem_rows,
                             stream>>>(in, (long long)ny * nx, my, mx, pad, work, P, lg, rpc, tw);
    fft_cols_kernel<<<dim3(P / cpc, (unsigned)n_inst), 256, 2 * smem_cols, stream>>>(
        work, my, work, wstride, P, lg, cpc, kspec, kstride == 0 ? 0 : (long long)P * P, keep0,
        ny, tw);
    fft_rows_inv_kernel<T><<<dim3((ny + rpc - 1) / rpc, (unsigned)n_inst), 256, smem_rows,
                             stream>>>(work, wstride, ny, out, (long long)ny * nx, nx, P, lg, rpc,
                                       keep0, 1.0 / ((double)P * P), tw);
    return 0;
}

int launch_conv_fft(const void* in, void* out, const void* kernel, long long kstride, int n_inst,
                    int ny, int nx, int K, int edge, int precision, void* scratch,
                    cudaStream_t stream) {
    if (n_inst <= 0) return 0;
    if (precision == LENSGB_FP64)
        return fft_conv_t<double>((const double*)in, (double*)out, (const double*)kernel,
                                  kstride, n_inst, ny, nx, K, edge, scratch, stream);
    return fft_conv_t<float>((const float*)in, (float*)out, (const float*)kernel, kstride, n_inst,
                             ny, nx, K, edge, scratch, stream);
}

}  // namespace lensgb
