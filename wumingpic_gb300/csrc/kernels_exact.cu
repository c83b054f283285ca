// FP64 kernels in the reference's operation order, compiled with -fmad=false
// (no fused multiply-add): the bit-exact parity build.
#include "common.cuh"

namespace wpic {
namespace exact {
#include "fp2d.cuh"
#include "fp3d.cuh"
}  // namespace exact
}  // namespace wpic
