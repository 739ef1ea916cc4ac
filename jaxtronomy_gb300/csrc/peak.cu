// FMA-chain kernel: measures the device's FP32 / FP64 fused multiply-add rate,
// the denominator of the roofline fractions of the ray-tracing and convolution
// kernels (all compute-bound on the FMA pipe; none is HBM- or tensor-bound).
//
// Each thread runs CHAINS independent dependency chains of `iters` FMAs
// x <- x * m + a, so every warp scheduler always has independent FMAs to
// issue; the chains' sum is written per thread so nothing is eliminated.
// FLOPs of one launch = blocks x 256 x CHAINS x iters x 2.
#include "launch.h"

namespace lensgb {

constexpr int PEAK_THREADS = 256, PEAK_CHAINS = 8;

template <typename R>
__global__ void __launch_bounds__(PEAK_THREADS) fma_chain_kernel(R m, R a, int iters, R* out) {
    R x[PEAK_CHAINS];
#pragma unroll
    for (int c = 0; c < PEAK_CHAINS; ++c) x[c] = (R)(threadIdx.x + c) * (R)1e-3;
    for (int i = 0; i < iters; i += 16) {
#pragma unroll
        for (int u = 0; u < 16; ++u)
#pragma unroll
            for (int c = 0; c < PEAK_CHAINS; ++c) x[c] = fma(x[c], m, a);
    }
    R sum = 0;
#pragma unroll
    for (int c = 0; c < PEAK_CHAINS; ++c) sum += x[c];
    out[(long long)blockIdx.x * PEAK_THREADS + threadIdx.x] = sum;
}

// The same chains on packed pairs (fma.rn.f32x2, one instruction for two FP32
// FMAs): 2 x PEAK_CHAINS chains per thread in PEAK_CHAINS pair registers.
__global__ void __launch_bounds__(PEAK_THREADS) fma2_chain_kernel(float m, float a, int iters,
                                                                  float* out) {
    float2 x[PEAK_CHAINS];
#pragma unroll
    for (int c = 0; c < PEAK_CHAINS; ++c)
        x[c] = make_float2((float)(threadIdx.x + c) * 1e-3f, (float)(threadIdx.x + c + 1) * 1e-3f);
    const float2 m2 = make_float2(m, m), a2 = make_float2(a, a);
    for (int i = 0; i < iters; i += 16) {
#pragma unroll
        for (int u = 0; u < 16; ++u)
#pragma unroll
            for (int c = 0; c < PEAK_CHAINS; ++c) x[c] = __ffma2_rn(x[c], m2, a2);
    }
    float sum = 0.f;
#pragma unroll
    for (int c = 0; c < PEAK_CHAINS; ++c) sum += x[c].x + x[c].y;
    out[(long long)blockIdx.x * PEAK_THREADS + threadIdx.x] = sum;
}

}  // namespace lensgb

using namespace lensgb;

extern "C" int lensgb_fma_chain(int precision, int blocks, int iters, void* out_dev,
                                long long* flops, void* stream) {
    if (blocks < 1 || iters < 16 || iters % 16 != 0 || !out_dev ||
        (precision != LENSGB_FP64 && precision != LENSGB_FP32_SPLIT &&
         precision != LENSGB_FP32_PAIRS)) {
        set_last_error("lensgb_fma_chain: a known precision, blocks >= 1, iters a positive "
                       "multiple of 16 and an output of blocks x 256 elements are required");
        return LENSGB_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    // m slightly below 1 keeps every chain finite for any iteration count
    if (precision == LENSGB_FP64)
        fma_chain_kernel<double><<<blocks, PEAK_THREADS, 0, s>>>(0.999999, 1e-6, iters,
                                                                 (double*)out_dev);
    else if (precision == LENSGB_FP32_SPLIT)
        fma_chain_kernel<float><<<blocks, PEAK_THREADS, 0, s>>>(0.9999f, 1e-4f, iters,
                                                                (float*)out_dev);
    else
        fma2_chain_kernel<<<blocks, PEAK_THREADS, 0, s>>>(0.9999f, 1e-4f, iters,
                                                          (float*)out_dev);
    if (flops)
        *flops = (long long)blocks * PEAK_THREADS * PEAK_CHAINS * iters * 2 *
                 (precision == LENSGB_FP32_PAIRS ? 2 : 1);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(std::string("lensgb_fma_chain launch: ") + cudaGetErrorString(e));
        return LENSGB_ERR_CUDA;
    }
    return LENSGB_OK;
}
