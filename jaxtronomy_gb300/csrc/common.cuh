// Shared definitions of the lens image kernels: per-profile parameter
// records, error-free FP32 transforms and small math helpers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/lensgb.h"

namespace lensgb {

// Derived per-(system, profile) record written by the prepare kernel.  Doubles
// serve the FP64 kernels and FP64 set-up; floats serve the FP32 kernels.
constexpr int REC_D = 32;
constexpr int REC_F = 36;  // float slot k + 2 mirrors double slot k >= 2
constexpr int TNFW_NC = 12;  // terms of the TNFW bracket polynomial (record slots d14..)
// EPL series coefficient table length (largest reference nmax, epl.py:311-319)
constexpr int EPL_NMAX = 500;
constexpr int MAX_PROF = LENSGB_MAX_PROFILES;

// Common record slots
//   d[0], d[1]           profile centre (center_x, center_y) or (ra_0, dec_0)
//   f[0..3]              FP32 split of the centre offset of the supersampled
//                        ray (0, 0):  X0 = ra(0,0) - cx = f0 + f1,
//                        Y0 = dec(0,0) - cy = f2 + f3
constexpr int RD_CX = 0, RD_CY = 1;
constexpr int RF_X0H = 0, RF_X0L = 1, RF_Y0H = 2, RF_Y0L = 3;

// Grid description shared by all kernels of one model.
struct GridDesc {
    int nx, ny, s;            // columns, rows, supersampling
    double ra00, dec00;       // coordinate of supersampled ray (0, 0)
    double ax, bx, ay, by;    // coordinate steps per supersampled column / row
    float ax_hi, ax_lo, bx_hi, bx_lo, ay_hi, ay_lo, by_hi, by_lo;
};

// Static description of the profile stack of a model.
struct StackDesc {
    int n_lens, n_src, n_ll;
    int lens[MAX_PROF];
    int src[MAX_PROF];
    int ll[MAX_PROF];
    int lens_off[MAX_PROF];   // column of each profile in a system row
    int src_off[MAX_PROF];
    int ll_off[MAX_PROF];
    int epl_slot[MAX_PROF];   // coefficient-table slot of each lens profile (-1: none):
                              // EPL series F_n, or the CSE term constants
    int n_epl;                // number of coefficient-table slots per system
    int n_params;
    double src_scale[MAX_PROF];  // deflection_scaling per source
    double alpha_scaling;
    double flux_scaling;
    // FP32 copies, so FP32 kernels never convert per ray
    float src_scale_f[MAX_PROF];
    float alpha_scaling_f;
    float flux_scaling_f;
};

// Pixels of the FP32 pass whose predicted error exceeds `tau` are appended to
// `list` (as system * nx * ny + pixel) and recomputed in FP64 by the refine pass.
struct RefineArgs {
    unsigned int* list;         // capacity: n_inst * nx * ny entries
    unsigned int* count;        // zeroed on the stream before the FP32 pass
    float tau;                  // tolerated predicted relative error per ray (<= 0: no refine)
    float kappa;                // FP32 relative error bound of |alpha| (units of 1)
};

// Launch over systems of different grids and supersampling factors (one
// model's profile stack).  Every table is per system, so its size does not
// depend on the pixel count, and the system counts are read on the device, so
// one launch configuration (e.g. a captured CUDA graph) serves batches of any
// mix.  The ray kernel runs once per supersampling group (FP32: s = 1..4 with
// the compile-time-s kernel, group 0 every other s; FP64: one group) -- so a
// system always runs the same instantiation, whatever shares its batch -- as a
// grid-stride loop over the group's tiles of 256 pixels: system sys[j] owns
// tiles tile_off[j] .. tile_off[j + 1] - 1.  grid == nullptr: a uniform launch
// (every system on the launch's own grid, images nx * ny apart).
struct MixedTab {
    const GridDesc* grid;     // [n]
    const long long* off;     // [n + 1]: element offset of each system's image
    const double* scale;      // [n]: image scale (pixel area) of each system
    const int* n_inst;        // device: n
    const int* sys;           // this launch's group: its systems, in order
    const int* tile_off;      // [count + 1]: first ray tile of each
    const int* count;         // device: systems in the group
    int s_group;              // host: the group's compile-time s (0: per system)
    bool refine;              // host: launch the refine pass after this group
};

// Convolution over systems of different sizes, one launch per kernel-width
// group: the group's systems sys[0 .. count-1] in order, conv tile prefix
// tile_off[0 .. count] (tiles of the kernel's tile size, row-major per
// system), and per system its grid (nx, ny), image offset, kernel offset and K.
// count == nullptr: a uniform launch.
struct ConvMixed {
    const GridDesc* grid;
    const long long* off;
    const long long* koff;
    const int* ksize;
    const int* sys;
    const int* tile_off;
    const int* count;
};

// Segment j of a strictly increasing prefix array off[0 .. n] with
// off[j] <= t < off[j + 1] (t < off[n]).
__device__ __forceinline__ int find_segment(const int* off, int n, int t) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(off + mid) <= t)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Unique profile codes of a bulk handle (LensModelBulk's unique_lens_model_list);
// index u.n stands for the NULL profile.
struct BulkUnique {
    int n;
    int code[LENSGB_BULK_MAX_UNIQUE];
};

// Per-deflector tag of a bulk call: profile code in the low byte, plus this
// flag when the deflector's terms run in FP64, and (multi-plane FP32 calls)
// the flag of a step that starts a new lens plane.
constexpr int BULK_TAG_FP64 = 0x100;
constexpr int BULK_TAG_PLANE = 0x200;
constexpr int BULK_CODE_MASK = 0xff;

// ---------------------------------------------------------------------------
// FP32 error-free transforms (Knuth TwoSum, Dekker split)
// ---------------------------------------------------------------------------

__device__ __forceinline__ float two_sum(float a, float b, float& err) {
    float s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return s;
}

// x - centre for the supersampled ray (I, J), as a float carrying the
// accuracy of an FP64 subtraction: the centre offset X0 is an FP64 value split
// into (hi, lo) floats, and J*a_hi is exact because a_hi has at most 12
// significant bits.
__device__ __forceinline__ float split_offset(float x0h, float x0l, float p_exact, float p_small) {
    float e;
    float s = two_sum(x0h, p_exact, e);
    return __fadd_rn(s, __fadd_rn(e, __fadd_rn(x0l, p_small)));
}

// Host/device: split an FP64 value into a float with at most `bits`
// significant bits and the float remainder.
__host__ __device__ inline void split_bits(double v, int bits, float& hi, float& lo) {
    if (v == 0.0) { hi = 0.f; lo = 0.f; return; }
    int e;
    double m = frexp(v, &e);                 // v = m * 2^e, 0.5 <= |m| < 1
    double scale = ldexp(1.0, bits);
    double mh = trunc(m * scale) / scale;    // keep `bits` bits
    double h = ldexp(mh, e);
    hi = (float)h;
    lo = (float)(v - h);
}

__host__ __device__ inline void split_double(double v, float& hi, float& lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

// Hardware approximations (PTX lg2.approx / ex2.approx, flush-to-zero, relative
// error about 2^-22).  The FP32 path uses them for the EPL power law and the
// Sersic profile; the resulting image error is measured against FP64 and the
// ill-conditioned rays are recomputed in FP64 anyway.
__device__ __forceinline__ float lg2_approx(float x) {
    float r;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float ex2_approx(float x) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// nan_to_num(posinf=1e10, neginf=-1e10), as used at epl.py:391-392
template <typename R>
__device__ __forceinline__ R nan_to_num_1e10(R v) {
    if (isnan(v)) return R(0);
    if (isinf(v)) return v > 0 ? R(1e10) : R(-1e10);
    return v;
}

// nan_to_num() with NumPy defaults, as used at sersic_utils.py:267
template <typename R>
__device__ __forceinline__ R nan_to_num_max(R v) {
    if (isnan(v)) return R(0);
    if (isinf(v)) return v > 0 ? (sizeof(R) == 8 ? R(1.7976931348623157e308) : R(3.4028234663852886e38))
                               : (sizeof(R) == 8 ? R(-1.7976931348623157e308) : R(-3.4028234663852886e38));
    return v;
}

}  // namespace lensgb
