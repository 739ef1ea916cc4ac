// Ray-tracing kernels specialised for NFW_ELLIPSE_CSE + SHEAR lens stacks.
#include "raytrace_kernels.cuh"

namespace lensgb {
LENSGB_DEFINE_VARIANT(LENSGB_LENS_NFW_ELLIPSE_CSE, LENSGB_LENS_SHEAR, 1, 1)
LENSGB_DEFINE_VARIANT(LENSGB_LENS_NFW_ELLIPSE_CSE, LENSGB_LENS_SHEAR, 2, 1)
}  // namespace lensgb
