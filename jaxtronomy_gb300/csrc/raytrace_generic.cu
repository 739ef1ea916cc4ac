// Generic ray-tracing kernels: any lens stack, walked at run time.
#include "raytrace_kernels.cuh"

namespace lensgb {
LENSGB_DEFINE_VARIANT(GENERIC, 0, -1, -1)
}  // namespace lensgb
