// Ray-tracing kernels specialised for SIE + SHEAR lens stacks.
#include "raytrace_kernels.cuh"

namespace lensgb {
LENSGB_DEFINE_VARIANT(LENSGB_LENS_SIE, LENSGB_LENS_SHEAR, 1, 1)
LENSGB_DEFINE_VARIANT(LENSGB_LENS_SIE, LENSGB_LENS_SHEAR, 2, 1)
}  // namespace lensgb
