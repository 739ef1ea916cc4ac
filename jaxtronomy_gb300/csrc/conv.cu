// Direct "same"-mode 2-D PSF convolution with a shared-memory halo tile.
//
// Replaces PixelKernelConvolution.convolution2d (fftconvolve / convolve2d,
// "same" mode, zero boundary; JAXtronomy ImSim/Numerics/convolution.py:74-86)
// and the edge-padded GaussianConvolution.convolution2d (convolution.py:215-235).
// For odd K with h = K/2:
//   out[y][x] = sum_{u,v} ker[K-1-u][K-1-v] * in[y+u-h][x+v-h]
// with in[] = 0 outside the image (zero padding) or clamped to the nearest edge
// pixel (edge padding).
//
// Each CTA computes a TILE_H x TILE_W output tile of one system; the flipped
// kernel and the (TILE_H+K-1) x (TILE_W+KP-1) input halo tile sit in shared
// memory.  Each thread accumulates an RY x CX register block, streaming one
// input row segment at a time through registers and reusing it for every
// output row of its block that the row touches.
#include <cuda.h>  // CUtensorMap and its encoder's types (the encoder is fetched at run time)

#include <map>
#include <mutex>
#include <type_traits>
#include <utility>

#include "launch.h"

namespace lensgb {

constexpr int CONV_TX = 8, CONV_TY = 16;

// Which system and tile a CTA convolves.  Each kernel's body is a lambda
// tile(bxi, byi, nx, ny, K, ioff, koff) over one output tile; a uniform launch
// (MIXED = false) runs it once for tile (blockIdx.x, blockIdx.y) of system
// blockIdx.z.  Its arguments pass through an empty asm statement, so that the
// compiler schedules the body for opaque register values rather than for
// values it derives from blockIdx (measured on GB300: 1.35 -> 1.27 ms for
// 1024 images of 180^2 with K = 31).  A launch over systems of different sizes
// (MIXED = true) runs a grid-stride loop over the group's tiles, taking ny, nx,
// K and the image / kernel offsets from the per-system tables, with a barrier
// before the next tile refills shared memory.
#define CONV_RUN_TILES(TILE_W)                                                         \
    if (!MIXED) {                                                                      \
        int bxi = blockIdx.x, byi = blockIdx.y, nx_ = nx, ny_ = ny, K_ = K;            \
        long long ioff = (long long)blockIdx.z * ny * nx;                              \
        long long koff = (long long)blockIdx.z * kstride;                              \
        asm volatile("" : "+r"(bxi), "+r"(byi), "+r"(nx_), "+r"(ny_), "+r"(K_),        \
                     "+l"(ioff), "+l"(koff));                                          \
        tile(bxi, byi, nx_, ny_, K_, ioff, koff);                                      \
    } else {                                                                           \
        const int n_sys = *cm.count;                                                   \
        const int n_tiles = __ldg(cm.tile_off + n_sys);                                \
        for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {                        \
            const int j = find_segment(cm.tile_off, n_sys, t);                         \
            const int sys = __ldg(cm.sys + j);                                         \
            const int mx = cm.grid[sys].nx, my = cm.grid[sys].ny;                      \
            const int tx = (mx + (TILE_W) - 1) / (TILE_W);                             \
            const int l = t - __ldg(cm.tile_off + j);                                  \
            const int by = l / tx;                                                     \
            tile(l - by * tx, by, mx, my, __ldg(cm.ksize + sys), __ldg(cm.off + sys),  \
                 __ldg(cm.koff + sys));                                                \
            __syncthreads();                                                           \
        }                                                                              \
    }

template <typename R, int CX, int RY, int VC, bool MIXED>
__global__ void __launch_bounds__(CONV_TX* CONV_TY)
conv_kernel(const R* __restrict__ in, R* __restrict__ out, const R* __restrict__ ker,
            long long kstride, int ny, int nx, int K, int edge, ConvMixed cm) {
    constexpr int W = CONV_TX * CX, H = CONV_TY * RY;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto tile = [&](int bxi, int byi, int nx, int ny, int K, long long ioff, long long koff) {
        R* sk = (R*)smem_raw;
        const int KP = ((K + VC - 1) / VC) * VC;
        const int SW = W + KP - 1 + 1;  // +1 keeps row starts off the same bank
        const int SH = H + K - 1;
        R* si = sk + K * KP;
        const int ox0 = bxi * W, oy0 = byi * H;
        const int h = K / 2;
        const int tid = threadIdx.y * CONV_TX + threadIdx.x;
        const int nthr = CONV_TX * CONV_TY;
        const R* kk = ker + koff;
        for (int e = tid; e < K * KP; e += nthr) {
            int u = e / KP, v = e - u * KP;
            sk[e] = v < K ? kk[(K - 1 - u) * K + (K - 1 - v)] : R(0);
        }
        const R* img = in + ioff;
        for (int e = tid; e < SH * SW; e += nthr) {
            int r = e / SW, c = e - r * SW;
            int gy = oy0 - h + r, gx = ox0 - h + c;
            R v;
            if (edge) {
                gy = gy < 0 ? 0 : (gy >= ny ? ny - 1 : gy);
                gx = gx < 0 ? 0 : (gx >= nx ? nx - 1 : gx);
                v = img[(long long)gy * nx + gx];
            } else {
                v = (gy >= 0 && gy < ny && gx >= 0 && gx < nx) ? img[(long long)gy * nx + gx] : R(0);
            }
            si[e] = v;
        }
        __syncthreads();

        R acc[RY][CX];
#pragma unroll
        for (int i = 0; i < RY; ++i)
#pragma unroll
            for (int c = 0; c < CX; ++c) acc[i][c] = 0;
        const int c0 = threadIdx.x * CX, r0 = threadIdx.y * RY;
        for (int ir = 0; ir < RY + K - 1; ++ir) {
            const R* row = si + (r0 + ir) * SW + c0;
            for (int v0 = 0; v0 < KP; v0 += VC) {
                R seg[CX + VC - 1];
#pragma unroll
                for (int j = 0; j < CX + VC - 1; ++j) seg[j] = row[v0 + j];
#pragma unroll
                for (int i = 0; i < RY; ++i) {
                    const int u = ir - i;
                    if (u < 0 || u >= K) continue;
                    const R* kr = sk + u * KP + v0;
#pragma unroll
                    for (int vv = 0; vv < VC; ++vv) {
                        const R w = kr[vv];
#pragma unroll
                        for (int c = 0; c < CX; ++c) acc[i][c] = fma(w, seg[c + vv], acc[i][c]);
                    }
                }
            }
        }
        R* o = out + ioff;
#pragma unroll
        for (int i = 0; i < RY; ++i) {
            const int y = oy0 + r0 + i;
            if (y >= ny) continue;
#pragma unroll
            for (int c = 0; c < CX; ++c) {
                const int x = ox0 + c0 + c;
                if (x < nx) o[(long long)y * nx + x] = acc[i][c];
            }
        }
    };
    CONV_RUN_TILES(W)
}

// FP32 variant: each thread owns 4 rows x 8 columns; input segments and kernel
// rows come from shared memory as float4 (kernel rows zero-padded to KP, a
// multiple of 8).  blockDim = (8, TY) with TY chosen per image height so that
// the 4*TY-row tiles waste as few rows as possible.
constexpr int C32_CX = 8, C32_RY = 4, C32_TX = 8, C32_W = C32_TX * C32_CX;

template <bool MIXED>
__global__ void __launch_bounds__(C32_TX * 16)
conv_f32_kernel(const float* __restrict__ in, float* __restrict__ out,
                const float* __restrict__ ker, long long kstride, int ny, int nx, int K, int edge,
                ConvMixed cm) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto tile = [&](int bxi, int byi, int nx, int ny, int K, long long ioff, long long koff) {
        const int TY = blockDim.y;
        const int H = TY * C32_RY;
        const int KP = ((K + 7) / 8) * 8;
        const int SW = C32_W + KP + 4;  // multiple of 4 floats: rows stay 16-byte aligned
        const int SH = H + K - 1;
        float* sk = (float*)smem_raw;
        float* si = sk + K * KP;
        const int ox0 = bxi * C32_W, oy0 = byi * H;
        const int h = K / 2;
        const int tid = threadIdx.y * C32_TX + threadIdx.x;
        const int nthr = C32_TX * TY;
        const float* kk = ker + koff;
        for (int e = tid; e < K * KP; e += nthr) {
            const int u = e / KP, v = e - u * KP;
            sk[e] = v < K ? kk[(K - 1 - u) * K + (K - 1 - v)] : 0.f;
        }
        const float* img = in + ioff;
        for (int e = tid; e < SH * SW; e += nthr) {
            const int r = e / SW, c = e - r * SW;
            int gy = oy0 - h + r, gx = ox0 - h + c;
            float v;
            if (edge) {
                gy = gy < 0 ? 0 : (gy >= ny ? ny - 1 : gy);
                gx = gx < 0 ? 0 : (gx >= nx ? nx - 1 : gx);
                v = img[(long long)gy * nx + gx];
            } else {
                v = (gy >= 0 && gy < ny && gx >= 0 && gx < nx) ? img[(long long)gy * nx + gx] : 0.f;
            }
            si[e] = v;
        }
        __syncthreads();

        float acc[C32_RY][C32_CX];
#pragma unroll
        for (int i = 0; i < C32_RY; ++i)
#pragma unroll
            for (int c = 0; c < C32_CX; ++c) acc[i][c] = 0.f;
        const int c0 = threadIdx.x * C32_CX, r0 = threadIdx.y * C32_RY;
        for (int ir = 0; ir < C32_RY + K - 1; ++ir) {
            const float4* row = reinterpret_cast<const float4*>(si + (r0 + ir) * SW + c0);
            for (int v0 = 0; v0 < KP; v0 += 8) {
                float seg[16];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const float4 q = row[v0 / 4 + j];
                    seg[4 * j] = q.x;
                    seg[4 * j + 1] = q.y;
                    seg[4 * j + 2] = q.z;
                    seg[4 * j + 3] = q.w;
                }
#pragma unroll
                for (int i = 0; i < C32_RY; ++i) {
                    const int u = ir - i;
                    if (u < 0 || u >= K) continue;
                    const float4* kr = reinterpret_cast<const float4*>(sk + u * KP + v0);
                    const float4 k0 = kr[0], k1 = kr[1];
                    const float w[8] = {k0.x, k0.y, k0.z, k0.w, k1.x, k1.y, k1.z, k1.w};
#pragma unroll
                    for (int vv = 0; vv < 8; ++vv)
#pragma unroll
                        for (int c = 0; c < C32_CX; ++c) acc[i][c] = fmaf(w[vv], seg[c + vv], acc[i][c]);
                }
            }
        }
        float* o = out + ioff;
#pragma unroll
        for (int i = 0; i < C32_RY; ++i) {
            const int y = oy0 + r0 + i;
            if (y >= ny) continue;
#pragma unroll
            for (int c = 0; c < C32_CX; ++c) {
                const int x = ox0 + c0 + c;
                if (x < nx) o[(long long)y * nx + x] = acc[i][c];
            }
        }
    };
    CONV_RUN_TILES(C32_W)
}

// The compute of one thread's 4 x 8 output block of the fixed-width kernels:
// `base` is the halo tile at the block's first input row and column (row
// pitch 64 + 8 NSEG + 4 floats, 16-byte aligned), `sk` the flipped kernel
// rows zero-padded to 8 NSEG columns.  Every output sums its products in
// (kernel row, kernel column) order.
template <int NSEG>
__device__ __forceinline__ void conv_f32_fixed_tile(const float* base, const float* sk, int K,
                                                    float (&acc)[C32_RY][C32_CX]) {
    constexpr int KP = 8 * NSEG;
    constexpr int SW = C32_W + KP + 4;
#pragma unroll
    for (int i = 0; i < C32_RY; ++i)
#pragma unroll
        for (int c = 0; c < C32_CX; ++c) acc[i][c] = 0.f;
    // input row ir feeds output row i through kernel row ir - i
    auto row_step = [&](int ir, int ilo, int ihi) {
        const float4* row = reinterpret_cast<const float4*>(base + ir * SW);
#pragma unroll
        for (int sg = 0; sg < NSEG; ++sg) {
            float seg[16];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float4 q = row[2 * sg + j];
                seg[4 * j] = q.x;
                seg[4 * j + 1] = q.y;
                seg[4 * j + 2] = q.z;
                seg[4 * j + 3] = q.w;
            }
#pragma unroll
            for (int i = 0; i < C32_RY; ++i) {
                if (i < ilo || i > ihi) continue;
                const float4* kr = reinterpret_cast<const float4*>(sk + (ir - i) * KP + 8 * sg);
                const float4 k0 = kr[0], k1 = kr[1];
                const float w[8] = {k0.x, k0.y, k0.z, k0.w, k1.x, k1.y, k1.z, k1.w};
#pragma unroll
                for (int vv = 0; vv < 8; ++vv)
#pragma unroll
                    for (int c = 0; c < C32_CX; ++c) acc[i][c] = fmaf(w[vv], seg[c + vv], acc[i][c]);
            }
        }
    };
    // output row i takes input rows i .. i+K-1, i.e. input row ir serves the
    // output rows max(0, ir-K+1) .. min(RY-1, ir)
    // head: input rows 0 .. RY-2
    for (int ir = 0; ir < C32_RY - 1; ++ir)
        row_step(ir, ir - K + 1 > 0 ? ir - K + 1 : 0, ir);
    // body: rows RY-1 .. K-1 serve every output row (branch-free)
    for (int ir = C32_RY - 1; ir < K; ++ir) row_step(ir, 0, C32_RY - 1);
    // tail: rows max(K, RY-1) .. K+RY-2
    for (int ir = (K > C32_RY - 1 ? K : C32_RY - 1); ir < K + C32_RY - 1; ++ir)
        row_step(ir, ir - K + 1, C32_RY - 1);
}

// FP32 variant with the kernel width fixed at compile time (NSEG segments of 8
// columns, K <= 8 NSEG): the same tiles and shared-memory layout as
// conv_f32_kernel, but the input-row loop is split so that its middle part --
// every output row of the thread has a kernel row -- runs without branches and
// with all shared-memory offsets as immediates, and the halo tile is filled row
// by row without index divisions.
template <int NSEG, bool MIXED>
__global__ void __launch_bounds__(C32_TX * 16)
conv_f32_fixed_kernel(const float* __restrict__ in, float* __restrict__ out,
                      const float* __restrict__ ker, long long kstride, int ny, int nx, int K,
                      int edge, ConvMixed cm) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto tile = [&](int bxi, int byi, int nx, int ny, int K, long long ioff, long long koff) {
        constexpr int KP = 8 * NSEG;
        constexpr int SW = C32_W + KP + 4;  // multiple of 4 floats: rows stay 16-byte aligned
        const int TY = blockDim.y;
        const int H = TY * C32_RY;
        const int SH = H + K - 1;
        float* sk = (float*)smem_raw;
        float* si = sk + K * KP;
        const int ox0 = bxi * C32_W, oy0 = byi * H;
        const int h = K / 2;
        const int tid = threadIdx.y * C32_TX + threadIdx.x;
        const int nthr = C32_TX * TY;
        const float* kk = ker + koff;
        for (int e = tid; e < K * KP; e += nthr) {
            const int u = e / KP, v = e % KP;
            sk[e] = v < K ? kk[(K - 1 - u) * K + (K - 1 - v)] : 0.f;
        }
        const float* img = in + ioff;
        for (int r = threadIdx.y; r < SH; r += TY) {
            int gy = oy0 - h + r;
            const bool rin = gy >= 0 && gy < ny;
            if (edge) gy = gy < 0 ? 0 : (gy >= ny ? ny - 1 : gy);
            const float* grow = img + (long long)gy * nx;
            float* srow = si + r * SW;
            for (int c = threadIdx.x; c < SW; c += C32_TX) {
                int gx = ox0 - h + c;
                float v;
                if (edge) {
                    gx = gx < 0 ? 0 : (gx >= nx ? nx - 1 : gx);
                    v = grow[gx];
                } else {
                    v = (rin && gx >= 0 && gx < nx) ? grow[gx] : 0.f;
                }
                srow[c] = v;
            }
        }
        __syncthreads();

        float acc[C32_RY][C32_CX];
        const int c0 = threadIdx.x * C32_CX, r0 = threadIdx.y * C32_RY;
        conv_f32_fixed_tile<NSEG>(si + r0 * SW + c0, sk, K, acc);
        float* o = out + ioff;
#pragma unroll
        for (int i = 0; i < C32_RY; ++i) {
            const int y = oy0 + r0 + i;
            if (y >= ny) continue;
#pragma unroll
            for (int c = 0; c < C32_CX; ++c) {
                const int x = ox0 + c0 + c;
                if (x < nx) o[(long long)y * nx + x] = acc[i][c];
            }
        }
    };
    CONV_RUN_TILES(C32_W)
}

// Raise a kernel's dynamic shared-memory limit only when a launch needs more
// than any earlier one (per device and kernel), so that repeated launches --
// including ones recorded into a CUDA graph -- make no attribute calls.
static bool raise_smem_limit(const void* fn, size_t smem) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, size_t> granted;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(mu);
    size_t& g = granted[std::make_pair(fn, dev)];
    if (smem <= g) return true;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess) {
        cudaGetLastError();  // a refused size leaves no error behind for later calls
        return false;
    }
    g = smem;
    return true;
}

// ---------------------------------------------------------------------------
// TMA-staged halo tile (zero padding, uniform launches)
// ---------------------------------------------------------------------------
// The halo tile of conv_f32_fixed_kernel filled by one tensor-memory-
// accelerator copy per CTA: a 3-D tensor map over the batch (x = column,
// y = row, z = system) and one box of SW x SH floats.  The box's out-of-range
// elements -- negative coordinates included -- arrive as zeros, which is the
// zero padding of PixelKernelConvolution.  A tiled copy must start at an x
// coordinate that is a multiple of 4 floats (16 bytes); the halo starts at
// ox0 - h, so the box starts d = (ox0 - h) mod 4 columns to its left, and the
// kernel rows carry d leading zero columns instead: input column ox0 + c + v - h
// is tile column c + v + d, read against kernel column v + d.  Because
// ox0 is a multiple of 64, d depends only on K, and 8 NSEG >= K + d holds for
// every odd K, so no FMA is added; the non-zero products of every output are
// summed in the same order as in conv_f32_fixed_kernel, which therefore gives
// the same values bit for bit.
//
// The wait on the copy's mbarrier is bounded: after CONV_TMA_SPIN_LIMIT failed
// polls a CTA counts a timeout in g_conv_wait_timeouts (read by
// lensgb_wait_timeouts) and leaves without computing.
constexpr unsigned int CONV_TMA_SPIN_LIMIT = 1u << 22;
__device__ unsigned int g_conv_wait_timeouts = 0;

template <int NSEG>
__global__ void __launch_bounds__(C32_TX * 16)
conv_f32_tma_kernel(const __grid_constant__ CUtensorMap tmap, float* __restrict__ out,
                    const float* __restrict__ ker, long long kstride, int ny, int nx, int K,
                    int d) {
    constexpr int KP = 8 * NSEG;
    constexpr int SW = C32_W + KP + 4;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) unsigned long long bar;
    float* si = reinterpret_cast<float*>(
        (reinterpret_cast<size_t>(smem_raw) + 127) & ~static_cast<size_t>(127));
    // opaque launch values, as in CONV_RUN_TILES: the body is scheduled for
    // register values rather than for expressions of blockIdx
    int bxi = blockIdx.x, byi = blockIdx.y, bzi = blockIdx.z;
    asm volatile("" : "+r"(bxi), "+r"(byi), "+r"(bzi), "+r"(nx), "+r"(ny), "+r"(K), "+r"(d));
    const int TY = blockDim.y;
    const int H = TY * C32_RY;
    const int SH = H + K - 1;
    float* sk = si + SH * SW;
    const int ox0 = bxi * C32_W, oy0 = byi * H;
    const int h = K / 2;
    const int tid = threadIdx.y * C32_TX + threadIdx.x;
    const int nthr = C32_TX * TY;
    const unsigned int bar_s = static_cast<unsigned int>(__cvta_generic_to_shared(&bar));
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_s));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const unsigned int bytes = static_cast<unsigned int>(SH * SW * sizeof(float));
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_s),
                     "r"(bytes)
                     : "memory");
        const int x = ox0 - h - d, y = oy0 - h, z = bzi;
        const unsigned int dst = static_cast<unsigned int>(__cvta_generic_to_shared(si));
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
            " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
            "l"(reinterpret_cast<unsigned long long>(&tmap)), "r"(x), "r"(y), "r"(z),
            "r"(bar_s)
            : "memory");
    }
    // the flipped kernel, shifted right by d zero columns, while the copy runs
    const float* kk = ker + (long long)bzi * kstride;
    for (int e = tid; e < K * KP; e += nthr) {
        const int u = e / KP, v = e % KP - d;
        sk[e] = (v >= 0 && v < K) ? kk[(K - 1 - u) * K + (K - 1 - v)] : 0.f;
    }
    __syncthreads();  // kernel rows written; the barrier is initialised
    unsigned int done = 0;
    for (unsigned int it = 0; it < CONV_TMA_SPIN_LIMIT && !done; ++it) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(bar_s)
            : "memory");
    }
    if (!done) {
        if (tid == 0) atomicAdd(&g_conv_wait_timeouts, 1u);
        return;
    }
    float acc[C32_RY][C32_CX];
    const int c0 = threadIdx.x * C32_CX, r0 = threadIdx.y * C32_RY;
    conv_f32_fixed_tile<NSEG>(si + r0 * SW + c0, sk, K, acc);
    float* o = out + (long long)bzi * ny * nx;
#pragma unroll
    for (int i = 0; i < C32_RY; ++i) {
        const int y = oy0 + r0 + i;
        if (y >= ny) continue;
#pragma unroll
        for (int c = 0; c < C32_CX; ++c) {
            const int x = ox0 + c0 + c;
            if (x < nx) o[(long long)y * nx + x] = acc[i][c];
        }
    }
}

static int g_conv_tma = 1;  // lensgb_set_conv_tma

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        cudaGetLastError();
    });
    return fn;
}

// The TMA path of run_conv_f32: returns 1 when it does not apply (edge padding,
// a row pitch that is not a multiple of 16 bytes, an unaligned base, a kernel
// wider than the compile-time widths, a box above 256 rows or columns, or no
// tensor-map encoder), 0 when launched, -1 on a configuration error.
static int run_conv_f32_tma(const float* in, float* out, const float* kernel, long long kstride,
                            int n_inst, int ny, int nx, int K, int TY, cudaStream_t stream) {
    const int h = K / 2;
    const int d = ((-h) % 4 + 4) % 4;
    const int KP = ((K + d + 7) / 8) * 8;
    const int NSEG = KP / 8;
    const int SW = C32_W + KP + 4, H = 4 * TY, SH = H + K - 1;
    if (!g_conv_tma || NSEG > 6 || nx % 4 != 0 || (reinterpret_cast<size_t>(in) & 15) ||
        SW > 256 || SH > 256)
        return 1;
    EncodeTiledFn enc = encode_tiled();
    if (!enc) return 1;
    CUtensorMap tmap;
    const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)n_inst};
    const cuuint64_t strides[2] = {(cuuint64_t)nx * 4, (cuuint64_t)nx * ny * 4};
    const cuuint32_t box[3] = {(cuuint32_t)SW, (cuuint32_t)SH, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    if (enc(&tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(in), dims, strides, box,
            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return 1;
    const size_t smem = (size_t)(SH * SW + K * KP) * sizeof(float) + 128;
    const dim3 grid((unsigned)((nx + C32_W - 1) / C32_W), (unsigned)((ny + H - 1) / H),
                    (unsigned)n_inst);
    const dim3 block(C32_TX, TY);
    auto go = [&](auto nseg_tag) {
        constexpr int NS = decltype(nseg_tag)::value;
        const void* fn = (const void*)conv_f32_tma_kernel<NS>;
        if (smem > 48 * 1024 && !raise_smem_limit(fn, smem)) return -1;
        conv_f32_tma_kernel<NS><<<grid, block, smem, stream>>>(tmap, out, kernel, kstride, ny, nx,
                                                               K, d);
        return 0;
    };
    switch (NSEG) {
        case 1: return go(std::integral_constant<int, 1>());
        case 2: return go(std::integral_constant<int, 2>());
        case 3: return go(std::integral_constant<int, 3>());
        case 4: return go(std::integral_constant<int, 4>());
        case 5: return go(std::integral_constant<int, 5>());
        case 6: return go(std::integral_constant<int, 6>());
        default: return 1;
    }
}

static int run_conv_f32(const void* in, void* out, const void* kernel, long long kstride,
                        int n_inst, int ny, int nx, int K, int edge, cudaStream_t stream,
                        int tile_rows) {
    // tile height 4*TY with TY in 8..16: a tuned choice, else fewest padded
    // rows, then the tallest tile
    int best_ty = 16;
    long long best_waste = -1;
    for (int ty = 16; ty >= 8; --ty) {
        const int H = 4 * ty;
        const long long waste = (long long)((ny + H - 1) / H) * H - ny;
        if (best_waste < 0 || waste < best_waste) {
            best_waste = waste;
            best_ty = ty;
        }
    }
    if (tile_rows >= 32 && tile_rows <= 64 && tile_rows % 4 == 0) best_ty = tile_rows / 4;
    if (!edge) {
        const int r = run_conv_f32_tma((const float*)in, (float*)out, (const float*)kernel,
                                       kstride, n_inst, ny, nx, K, best_ty, stream);
        if (r <= 0) return r;
    }
    const int H = 4 * best_ty;
    const int KP = ((K + 7) / 8) * 8;
    const int SW = C32_W + KP + 4;
    const int SH = H + K - 1;
    const size_t smem = (size_t)(K * KP + SH * SW) * sizeof(float);
    dim3 grid((unsigned)((nx + C32_W - 1) / C32_W), (unsigned)((ny + H - 1) / H), (unsigned)n_inst);
    dim3 block(C32_TX, best_ty);
    const float* fin = (const float*)in;
    const float* fk = (const float*)kernel;
    auto fixed = [&](auto nseg_tag) {
        constexpr int NS = decltype(nseg_tag)::value;
        const void* fn = (const void*)conv_f32_fixed_kernel<NS, false>;
        if (smem > 48 * 1024 && !raise_smem_limit(fn, smem)) return -1;
        conv_f32_fixed_kernel<NS, false><<<grid, block, smem, stream>>>(
            fin, (float*)out, fk, kstride, ny, nx, K, edge, ConvMixed{});
        return 0;
    };
    switch (KP / 8) {
        case 1: return fixed(std::integral_constant<int, 1>());
        case 2: return fixed(std::integral_constant<int, 2>());
        case 3: return fixed(std::integral_constant<int, 3>());
        case 4: return fixed(std::integral_constant<int, 4>());
        case 5: return fixed(std::integral_constant<int, 5>());
        case 6: return fixed(std::integral_constant<int, 6>());
        default: break;
    }
    if (smem > 48 * 1024 && !raise_smem_limit((const void*)conv_f32_kernel<false>, smem)) return -1;
    conv_f32_kernel<false><<<grid, block, smem, stream>>>(fin, (float*)out, fk, kstride, ny, nx, K,
                                                          edge, ConvMixed{});
    return 0;
}

template <typename R, int CX, int RY, int VC>
static int run_conv(const void* in, void* out, const void* kernel, long long kstride, int n_inst,
                    int ny, int nx, int K, int edge, cudaStream_t stream) {
    constexpr int W = CONV_TX * CX, H = CONV_TY * RY;
    const int KP = ((K + VC - 1) / VC) * VC;
    const int SW = W + KP - 1 + 1;
    const int SH = H + K - 1;
    size_t smem = (size_t)(K * KP + SH * SW) * sizeof(R);
    if (smem > 48 * 1024 && !raise_smem_limit((const void*)conv_kernel<R, CX, RY, VC, false>, smem))
        return -1;
    dim3 grid((unsigned)((nx + W - 1) / W), (unsigned)((ny + H - 1) / H), (unsigned)n_inst);
    dim3 block(CONV_TX, CONV_TY);
    conv_kernel<R, CX, RY, VC, false><<<grid, block, smem, stream>>>(
        (const R*)in, (R*)out, (const R*)kernel, kstride, ny, nx, K, edge, ConvMixed{});
    return 0;
}

template <typename R>
__global__ void resize_kernel(const R* __restrict__ hr, R* __restrict__ out, int ny, int nx,
                              int s, double scale, int n_inst) {
    const long long npix = (long long)nx * ny;
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= npix * n_inst) return;
    const long long inst = gid / npix, p = gid % npix;
    const int row = (int)(p / nx), col = (int)(p % nx);
    const long long W = (long long)nx * s;
    const R* src = hr + inst * npix * s * s;
    double acc = 0.0;
    for (int si = 0; si < s; ++si) {
        double rs = 0.0;
        const R* r = src + ((long long)row * s + si) * W + (long long)col * s;
        for (int sj = 0; sj < s; ++sj) rs += (double)r[sj];
        acc += rs / (double)s;
    }
    out[gid] = (R)(acc / (double)s * scale);
}

int launch_resize(const void* hr, void* out, int n_inst, int ny, int nx, int s, double scale,
                  int precision, cudaStream_t stream) {
    const long long n = (long long)nx * ny * n_inst;
    if (n <= 0) return 0;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    if (precision == LENSGB_FP64)
        resize_kernel<double><<<blocks, 256, 0, stream>>>((const double*)hr, (double*)out, ny, nx,
                                                          s, scale, n_inst);
    else
        resize_kernel<float><<<blocks, 256, 0, stream>>>((const float*)hr, (float*)out, ny, nx, s,
                                                         scale, n_inst);
    return 0;
}

template <typename R>
__global__ void mask_kernel(R* __restrict__ img, long long n, int W, int s, int nx,
                            const unsigned char* __restrict__ mask, long long per_inst) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long p = i % per_inst;
    const int r = (int)(p / W), c = (int)(p % W);
    if (!mask[(long long)(r / s) * nx + c / s]) img[i] = (R)0;
}

int launch_mask(void* img, int n_inst, int ny, int nx, int s, const unsigned char* mask,
                int precision, cudaStream_t stream) {
    const long long per = (long long)ny * s * nx * s;
    const long long n = per * n_inst;
    if (n <= 0) return 0;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    if (precision == LENSGB_FP64)
        mask_kernel<double><<<blocks, 256, 0, stream>>>((double*)img, n, nx * s, s, nx, mask, per);
    else
        mask_kernel<float><<<blocks, 256, 0, stream>>>((float*)img, n, nx * s, s, nx, mask, per);
    return 0;
}

template <typename R>
__global__ void embed_kernel(const R* __restrict__ sub, R* __restrict__ out, long long n, int nsub,
                             int r0, int c0, int nyf, int nxf) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long per = (long long)nyf * nxf;
    const long long inst = i / per, p = i % per;
    const int r = (int)(p / nxf) - r0, c = (int)(p % nxf) - c0;
    out[i] = (r >= 0 && r < nsub && c >= 0 && c < nsub)
                 ? sub[(inst * nsub + r) * (long long)nsub + c]
                 : (R)0;
}

int launch_embed(const void* sub, void* out, int n_inst, int n, int r0, int c0, int ny_full,
                 int nx_full, int precision, cudaStream_t stream) {
    const long long total = (long long)ny_full * nx_full * n_inst;
    if (total <= 0) return 0;
    const unsigned blocks = (unsigned)((total + 255) / 256);
    if (precision == LENSGB_FP64)
        embed_kernel<double><<<blocks, 256, 0, stream>>>((const double*)sub, (double*)out, total, n,
                                                         r0, c0, ny_full, nx_full);
    else
        embed_kernel<float><<<blocks, 256, 0, stream>>>((const float*)sub, (float*)out, total, n,
                                                        r0, c0, ny_full, nx_full);
    return 0;
}

template <typename R>
__global__ void add_scaled_kernel(R* __restrict__ out, const R* __restrict__ add, long long n,
                                  double scale) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (R)(((double)out[i] + (double)add[i]) * scale);
}

int launch_add_scaled(void* out, const void* add, long long n, double scale, int precision,
                      cudaStream_t stream) {
    if (n <= 0) return 0;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    if (precision == LENSGB_FP64)
        add_scaled_kernel<double><<<blocks, 256, 0, stream>>>((double*)out, (const double*)add, n,
                                                              scale);
    else
        add_scaled_kernel<float><<<blocks, 256, 0, stream>>>((float*)out, (const float*)add, n,
                                                             scale);
    return 0;
}

int launch_conv_mixed(const void* in, void* out, const void* kernel, const ConvMixed& cm,
                      int n_ctas, int kmax, int group, int edge, int precision,
                      cudaStream_t stream) {
    if (n_ctas <= 0) return 0;
    const dim3 grid((unsigned)n_ctas);
    if (precision == LENSGB_FP64) {
        constexpr int W = CONV_TX * 4, H = CONV_TY * 4;
        const int KP = ((kmax + 3) / 4) * 4;
        const size_t smem = (size_t)(kmax * KP + (H + kmax - 1) * (W + KP)) * sizeof(double);
        const void* fn = (const void*)conv_kernel<double, 4, 4, 4, true>;
        if (smem > 48 * 1024 && !raise_smem_limit(fn, smem)) return -1;
        conv_kernel<double, 4, 4, 4, true><<<grid, dim3(CONV_TX, CONV_TY), smem, stream>>>(
            (const double*)in, (double*)out, (const double*)kernel, 0, 0, 0, 0, edge, cm);
        return 0;
    }
    // FP32: tiles of 64 x 64 (blockDim 8 x 16); `group` = kernel segments of 8
    // columns (0: the run-time-width kernel)
    const int TY = 16, H = 4 * TY;
    const int KP = group > 0 ? 8 * group : ((kmax + 7) / 8) * 8;
    const int SW = C32_W + KP + 4;
    const size_t smem = (size_t)(kmax * KP + (H + kmax - 1) * SW) * sizeof(float);
    const dim3 block(C32_TX, TY);
    const float* fin = (const float*)in;
    const float* fk = (const float*)kernel;
    auto fixed = [&](auto nseg_tag) {
        constexpr int NS = decltype(nseg_tag)::value;
        const void* fn = (const void*)conv_f32_fixed_kernel<NS, true>;
        if (smem > 48 * 1024 && !raise_smem_limit(fn, smem)) return -1;
        conv_f32_fixed_kernel<NS, true><<<grid, block, smem, stream>>>(
            fin, (float*)out, fk, 0, 0, 0, 0, edge, cm);
        return 0;
    };
    switch (group) {
        case 1: return fixed(std::integral_constant<int, 1>());
        case 2: return fixed(std::integral_constant<int, 2>());
        case 3: return fixed(std::integral_constant<int, 3>());
        case 4: return fixed(std::integral_constant<int, 4>());
        case 5: return fixed(std::integral_constant<int, 5>());
        case 6: return fixed(std::integral_constant<int, 6>());
        default: break;
    }
    if (smem > 48 * 1024 && !raise_smem_limit((const void*)conv_f32_kernel<true>, smem)) return -1;
    conv_f32_kernel<true><<<grid, block, smem, stream>>>(fin, (float*)out, fk, 0, 0, 0, 0, edge, cm);
    return 0;
}

bool direct_conv_fits(int K, int precision) {
    int dev = 0, limit = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&limit, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
            cudaSuccess ||
        limit <= 0) {
        cudaGetLastError();
        limit = 48 * 1024;
    }
    size_t smem;
    if (precision == LENSGB_FP64) {  // run_conv<double, 4, 4, 4>: 32 x 64 tiles
        const int KP = ((K + 3) / 4) * 4;
        smem = (size_t)(K * KP + (64 + K - 1) * (32 + KP)) * sizeof(double);
    } else {  // run_conv_f32 at its tallest tile (64 rows)
        const int KP = ((K + 7) / 8) * 8;
        smem = (size_t)(K * KP + (64 + K - 1) * (C32_W + KP + 4)) * sizeof(float);
    }
    return smem <= (size_t)limit;
}

void set_conv_tma(int enable) { g_conv_tma = enable ? 1 : 0; }

unsigned int conv_wait_timeouts() {
    unsigned int v = 0;
    cudaMemcpyFromSymbol(&v, g_conv_wait_timeouts, sizeof(v));
    return v;
}

int launch_conv(const void* in, void* out, const void* kernel, long long kstride, int n_inst,
                int ny, int nx, int K, int edge, int precision, cudaStream_t stream,
                int tile_rows) {
    if (precision == LENSGB_FP64) {
        // 32 x 64 tiles (4 x 4 outputs per thread); launches that would give
        // fewer than 2 CTAs per SM take 8 x 16 tiles (one output per thread).
        // Every output sums its K^2 products in the same (kernel row, kernel
        // column) order in both, so the two give identical values.
        const long long big = (long long)((nx + 31) / 32) * ((ny + 63) / 64) * n_inst;
        if (big < 2LL * num_sms())
            return run_conv<double, 1, 1, 4>(in, out, kernel, kstride, n_inst, ny, nx, K, edge,
                                             stream);
        return run_conv<double, 4, 4, 4>(in, out, kernel, kstride, n_inst, ny, nx, K, edge, stream);
    }
    return run_conv_f32(in, out, kernel, kstride, n_inst, ny, nx, K, edge, stream, tile_rows);
}

}  // namespace lensgb
