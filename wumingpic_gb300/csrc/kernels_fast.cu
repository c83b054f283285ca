// FP64 kernels with fused multiply-add contraction: the production FP64 build.
#include "common.cuh"

namespace wpic {
namespace fast {
#include "fp2d.cuh"
#include "fp3d.cuh"
}  // namespace fast
}  // namespace wpic
