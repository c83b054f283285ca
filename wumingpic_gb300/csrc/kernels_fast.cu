// FP64 kernels with fused multiply-add contraction: the production FP64 build.
#include "common.cuh"

namespace wpic {
namespace fast {
#define WPIC_REF_ORDER 0  // factored forms where they save FP64 operations (results within round-off)
#include "fp2d.cuh"
#include "fp3d.cuh"
#undef WPIC_REF_ORDER
}  // namespace fast
}  // namespace wpic
