// Ray-tracing kernels specialised for EPL_MULTIPOLE_M1M3M4 + SHEAR lens stacks.
#include "raytrace_kernels.cuh"

namespace lensgb {
LENSGB_DEFINE_VARIANT(LENSGB_LENS_EPL_MULTIPOLE_M1M3M4, LENSGB_LENS_SHEAR, 1, 1)
LENSGB_DEFINE_VARIANT(LENSGB_LENS_EPL_MULTIPOLE_M1M3M4, LENSGB_LENS_SHEAR, 2, 1)
}  // namespace lensgb
