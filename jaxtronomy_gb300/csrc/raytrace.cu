// Dispatch of the ray-tracing kernels (raytrace_kernels.cuh) to the profile
// stack of a model.  Common stacks run compile-time specialisations (their
// instantiations live in raytrace_epl.cu and raytrace_sie.cu so the build
// compiles them in parallel); every other stack runs the generic kernel
// (raytrace_generic.cu).
#include "raytrace_variants.h"

namespace lensgb {

int launch_raytrace(const GridDesc& g, const StackDesc& st, int n_inst, const double* rec_d,
                    const float* rec_f, const double* coef_d, const float* coef_f, void* out,
                    int flags, double out_scale, int precision, const RefineArgs& rf,
                    cudaStream_t stream, const MixedTab* mixed, int mixed_ctas, int ppt) {
    MixedTab mt;
    if (mixed) {
        mt = *mixed;
    } else {
        mt.grid = nullptr;
        mt.off = nullptr;
        mt.scale = nullptr;
        mt.n_inst = nullptr;
        mt.sys = nullptr;
        mt.tile_off = nullptr;
        mt.count = nullptr;
        mt.s_group = g.s;
        mt.refine = true;
    }
    const bool one_light = st.n_ll <= 1;
    const int a = st.n_lens == 2 ? st.lens[0] : 0, b = st.n_lens == 2 ? st.lens[1] : 0;
#define LENSGB_VARIANT(C0, C1, NS, NLL)                                                        \
    launch_variant<C0, C1, NS, NLL>(g, st, n_inst, rec_d, rec_f, coef_d, coef_f, out, flags, \
                                    out_scale, precision, rf, mt, mixed_ctas, ppt, stream)
    if (one_light && st.n_src >= 1 && st.n_src <= 2 && b == LENSGB_LENS_SHEAR) {
        if (a == LENSGB_LENS_EPL) {
            if (st.n_src == 1 && st.n_ll == 1) { LENSGB_VARIANT(LENSGB_LENS_EPL, LENSGB_LENS_SHEAR, 1, 1); return 0; }
            if (st.n_src == 2 && st.n_ll == 1) { LENSGB_VARIANT(LENSGB_LENS_EPL, LENSGB_LENS_SHEAR, 2, 1); return 0; }
            if (st.n_src == 1 && st.n_ll == 0) { LENSGB_VARIANT(LENSGB_LENS_EPL, LENSGB_LENS_SHEAR, 1, 0); return 0; }
        }
        if (a == LENSGB_LENS_SIE) {
            if (st.n_src == 1 && st.n_ll == 1) { LENSGB_VARIANT(LENSGB_LENS_SIE, LENSGB_LENS_SHEAR, 1, 1); return 0; }
            if (st.n_src == 2 && st.n_ll == 1) { LENSGB_VARIANT(LENSGB_LENS_SIE, LENSGB_LENS_SHEAR, 2, 1); return 0; }
        }
        if (a == LENSGB_LENS_EPL_MULTIPOLE_M1M3M4) {
            if (st.n_src == 1 && st.n_ll == 1) { LENSGB_VARIANT(LENSGB_LENS_EPL_MULTIPOLE_M1M3M4, LENSGB_LENS_SHEAR, 1, 1); return 0; }
            if (st.n_src == 2 && st.n_ll == 1) { LENSGB_VARIANT(LENSGB_LENS_EPL_MULTIPOLE_M1M3M4, LENSGB_LENS_SHEAR, 2, 1); return 0; }
        }
        if (a == LENSGB_LENS_NFW_ELLIPSE_CSE) {
            if (st.n_src == 1 && st.n_ll == 1) { LENSGB_VARIANT(LENSGB_LENS_NFW_ELLIPSE_CSE, LENSGB_LENS_SHEAR, 1, 1); return 0; }
            if (st.n_src == 2 && st.n_ll == 1) { LENSGB_VARIANT(LENSGB_LENS_NFW_ELLIPSE_CSE, LENSGB_LENS_SHEAR, 2, 1); return 0; }
        }
    }
    LENSGB_VARIANT(GENERIC, 0, -1, -1);
#undef LENSGB_VARIANT
    return 0;
}

}  // namespace lensgb
