// Explicitly instantiated ray-tracing launchers (one translation unit per
// group, so they compile in parallel).
#pragma once

#include "common.cuh"

namespace lensgb {

constexpr int GENERIC = -1;

template <int C0, int C1, int NS, int NLL>
void launch_variant(const GridDesc& g, const StackDesc& st, int n_inst, const double* rec_d,
                    const float* rec_f, const double* coef_d, const float* coef_f, void* out,
                    int flags, double out_scale, int precision, const RefineArgs& rf,
                    const MixedTab& mt, int mixed_ctas, int ppt, cudaStream_t stream);

#define LENSGB_DECLARE_VARIANT(C0, C1, NS, NLL)                                                 \
    extern template void launch_variant<C0, C1, NS, NLL>(                                      \
        const GridDesc&, const StackDesc&, int, const double*, const float*, const double*,    \
        const float*, void*, int, double, int, const RefineArgs&, const MixedTab&, int, int,   \
        cudaStream_t);
#define LENSGB_DEFINE_VARIANT(C0, C1, NS, NLL)                                                  \
    template void launch_variant<C0, C1, NS, NLL>(                                             \
        const GridDesc&, const StackDesc&, int, const double*, const float*, const double*,    \
        const float*, void*, int, double, int, const RefineArgs&, const MixedTab&, int, int,   \
        cudaStream_t);

LENSGB_DECLARE_VARIANT(LENSGB_LENS_EPL, LENSGB_LENS_SHEAR, 1, 1)
LENSGB_DECLARE_VARIANT(LENSGB_LENS_EPL, LENSGB_LENS_SHEAR, 2, 1)
LENSGB_DECLARE_VARIANT(LENSGB_LENS_EPL, LENSGB_LENS_SHEAR, 1, 0)
LENSGB_DECLARE_VARIANT(LENSGB_LENS_SIE, LENSGB_LENS_SHEAR, 1, 1)
LENSGB_DECLARE_VARIANT(LENSGB_LENS_SIE, LENSGB_LENS_SHEAR, 2, 1)
LENSGB_DECLARE_VARIANT(LENSGB_LENS_EPL_MULTIPOLE_M1M3M4, LENSGB_LENS_SHEAR, 1, 1)
LENSGB_DECLARE_VARIANT(LENSGB_LENS_EPL_MULTIPOLE_M1M3M4, LENSGB_LENS_SHEAR, 2, 1)
LENSGB_DECLARE_VARIANT(LENSGB_LENS_NFW_ELLIPSE_CSE, LENSGB_LENS_SHEAR, 1, 1)
LENSGB_DECLARE_VARIANT(LENSGB_LENS_NFW_ELLIPSE_CSE, LENSGB_LENS_SHEAR, 2, 1)
LENSGB_DECLARE_VARIANT(GENERIC, 0, -1, -1)

}  // namespace lensgb
