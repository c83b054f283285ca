// FP64 kernels in the reference's operation order, compiled with -fmad=false
// (no fused multiply-add): the bit-exact parity build.
#include "common.cuh"

namespace wpic {
namespace exact {
#define WPIC_REF_ORDER 1  // every FP64 expression in the reference's operation order
#include "fp2d.cuh"
#include "fp3d.cuh"
#undef WPIC_REF_ORDER
}  // namespace exact
}  // namespace wpic
