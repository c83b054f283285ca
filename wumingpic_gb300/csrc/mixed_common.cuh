// FP32 helpers shared by the mixed-precision 2D and 3D paths: the factored spline
// difference of the Esirkepov deposit and the exact two-plane fixed-point split used
// for shared-memory current sums.
#pragma once

namespace wpic {

// s1 - s0 of the quadratic spline over node offsets -2..2 of the old cell, in factored
// form.  o = old offset, p = new offset in the new cell, inc = new cell - old cell.
// Each entry is a product of small exact-ish factors (offset differences, distances to
// the cell faces) instead of a difference of O(1) spline values, so small displacements
// keep FP32 relative accuracy and Esirkepov's charge conservation holds to ~1e-7 in FP32.
// The three cases are evaluated and selected, so the warp does not diverge.
__device__ __forceinline__ void shape_diff5(float o, float p, int inc, float ds[5]) {
  const float dl = p - o, sp = o + p;
  const float z0 = -0.5f * dl * (2.f - sp), z1 = -dl * (sp - 1.f), z2 = 0.5f * dl * sp;
  const float qo = 1.f - o, qp = 1.f - p;
  const float a0 = -0.5f * qo * qo, a1 = -p * (1.f - 0.5f * p) - o * qo, a2 = p * qp + 0.5f * qo * (1.f + o),
              a3 = 0.5f * p * p;
  const float b0 = 0.5f * qp * qp, b1 = p * qp + o * (1.f - 0.5f * o), b2 = -0.5f * qp * (1.f + p) - o * qo,
              b3 = -0.5f * o * o;
  ds[0] = inc < 0 ? b0 : 0.f;
  ds[1] = inc == 0 ? z0 : (inc > 0 ? a0 : b1);
  ds[2] = inc == 0 ? z1 : (inc > 0 ? a1 : b2);
  ds[3] = inc == 0 ? z2 : (inc > 0 ? a2 : b3);
  ds[4] = inc > 0 ? a3 : 0.f;
}

// Two-plane fixed-point split of an FP32 contribution v: hi = round(v s1), lo = round((v - hi/s1) s2),
// with s2 = 2^15 s1.  Rounding by the magic-number addition (1.5 * 2^23): exact for |v s1| < 2^22,
// and v - hi/s1 is exact (Sterbenz), so hi/s1 + lo/s2 equals v to within 1/(2 s2).  Both planes are
// summed with native 32-bit shared-memory integer atomics: exact, hence order independent.
__device__ __forceinline__ void fx_add(int* hi, int* lo, float v, float s1, float is1, float s2) {
  const float M = 12582912.0f;  // 1.5 * 2^23
  const float t = fmaf(v, s1, M);
  const float hf = t - M;
  const float r = fmaf(-hf, is1, v);
  const float u = fmaf(r, s2, M);
  atomicAdd(hi, __float_as_int(t) - 0x4B400000);
  atomicAdd(lo, __float_as_int(u) - 0x4B400000);
}

}  // namespace wpic
