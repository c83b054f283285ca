// Mixed-precision 2D path: FP32 push, gather and deposition weights on
// integer-cell + FP32-offset positions; FP32 tile currents flushed into FP64
// global J; FP64 field state and solver (the FP64 kernels in fp2d.cuh).
//
// One CTA per 16 x 16-cell tile runs particle__solv and ele_cur fused
// (2d/common/particle.f90:48-179, 2d/common/field.f90:189-316): the tile's
// E/B stencil (20 x 20 nodes x 6 components, FP64) arrives in shared memory by
// one TMA tensor load, is averaged to cell centres in FP32, every particle of
// the tile's bins is pushed in place, and its Esirkepov current goes into an
// FP32 shared-memory tile that is added once into FP64 global J.  The periodic
// particle wraps of boundary_periodic__particle_x/_y are integer cell
// arithmetic here; the conducting-wall reflection of
// boundary_reconnection__particle_x is applied before the deposit, as in the
// reconnection driver's order.  Particles that leave their tile are then moved
// between bins by a deterministic two-kernel migration (holes filled in slot
// order from the arrivals, then from the bin's tail: the reference's scheme at
// tile granularity).
#include <cuda.h>

#include "common.cuh"

namespace wpic {

namespace {

constexpr int MP_THREADS = 256;
constexpr int TW = MIX_TS + 4;   // staged field nodes per tile edge (cells -2 .. 17)
constexpr int TT = MIX_TS + 2;   // cell-centred values per tile edge (cells -1 .. 16)
// Row pitch of the FP32 current tile.  The lanes of a warp sit in two consecutive cell rows
// (bins are filled round-robin over the 256 cells); a pitch of 16 (mod 32) words puts the
// two rows on disjoint banks, so the deposit atomics of such a warp are conflict-free.
constexpr int JP = 48;
constexpr unsigned long long kSpinLimit = 1ull << 22;  // a few seconds at most

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned phase) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}

// TMA: 3D tile (x = field column, y = field row, z = component) into shared memory
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* tm, int x, int y, int z,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(smem_u32(dst)), "l"(tm), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// bounded wait on phase 0 of the barrier; returns false if the limit was reached
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar) {
  for (unsigned long long it = 0; it < kSpinLimit; ++it)
    if (mbar_try_wait(bar, 0)) return true;
  return false;
}

__device__ __forceinline__ int dir_dx(int d) { return d % 3 - 1; }
__device__ __forceinline__ int dir_dy(int d) { return d / 3 - 1; }

// s1 - s0 of the quadratic spline on the 4-node window of the deposit, in factored form.
// o = old offset in the old cell, p = new offset in the new cell, inc = new cell - old cell.
// Written as products of small exact-ish factors (differences of offsets, distances to the
// cell faces) instead of differences of O(1) spline values, so each entry keeps FP32
// relative accuracy for small displacements: Esirkepov's charge conservation then holds to
// ~1e-7 relative in FP32.  Window: offsets -1..2 (inc >= 0) or -2..1 (inc < 0).
__device__ __forceinline__ void shape_diff(float o, float p, int inc, float ds[4]) {
  // the three cases are evaluated and selected, so the warp does not diverge
  const float dl = p - o, sp = o + p;
  const float z0 = -0.5f * dl * (2.f - sp), z1 = -dl * (sp - 1.f), z2 = 0.5f * dl * sp;
  const float qo = 1.f - o, qp = 1.f - p;
  const float a0 = -0.5f * qo * qo, a1 = -p * (1.f - 0.5f * p) - o * qo, a2 = p * qp + 0.5f * qo * (1.f + o),
              a3 = 0.5f * p * p;
  const float b0 = 0.5f * qp * qp, b1 = p * qp + o * (1.f - 0.5f * o), b2 = -0.5f * qp * (1.f + p) - o * qo,
              b3 = -0.5f * o * o;
  ds[0] = inc == 0 ? z0 : (inc > 0 ? a0 : b0);
  ds[1] = inc == 0 ? z1 : (inc > 0 ? a1 : b1);
  ds[2] = inc == 0 ? z2 : (inc > 0 ? a2 : b2);
  ds[3] = inc == 0 ? 0.f : (inc > 0 ? a3 : b3);
}

}  // namespace

int mix_make_tensor_map(const Dev2D& d, void* out) {
  typedef CUresult (*EncodeFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                               const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                               CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn)
    return -1;
  const cuuint64_t dims[3] = {(cuuint64_t)d.g.fp, (cuuint64_t)(d.g.ny + 4), 6};
  const cuuint64_t strides[2] = {(cuuint64_t)d.g.fp * sizeof(double), (cuuint64_t)d.g.fplane * sizeof(double)};
  const cuuint32_t box[3] = {TW, TW, 6};
  const cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = ((EncodeFn)fn)((CUtensorMap*)out, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, d.uf, dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : -2;
}

// ---------------------------------------------------------------------------
// fused push + deposit, one CTA per tile
// ---------------------------------------------------------------------------
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

__global__ void __launch_bounds__(MP_THREADS, 4) k_mix_push(Dev2D d, const __grid_constant__ CUtensorMap tm) {
  // the TMA staging of uf is dead once the cell-centred values exist; its bytes then hold the
  // fixed-point current planes of the tile
  __shared__ __align__(128) unsigned char sbuf[(6 * TW * TW * 8 > 2 * 3 * TW * JP * 4) ? 6 * TW * TW * 8
                                                                                     : 2 * 3 * TW * JP * 4];
  double(*suf)[TW][TW] = reinterpret_cast<double(*)[TW][TW]>(sbuf);
  int(*jhi)[TW][JP] = reinterpret_cast<int(*)[TW][JP]>(sbuf);
  int(*jlo)[TW][JP] = reinterpret_cast<int(*)[TW][JP]>(sbuf + 3 * TW * JP * 4);
  __shared__ __align__(16) float2 stmp[3][TT * TT];  // (Bx,By), (Bz,Ex), (Ey,Ez) at cell centres
  __shared__ __align__(8) unsigned long long bar;
  const Mix2D& m = d.m;
  const int tile = blockIdx.x;
  const int tx = tile % m.ntx, ty = tile / m.ntx;
  const Grid2D g = d.g;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_expect_tx(&bar, (unsigned)(6 * TW * TW * sizeof(double)));
    tma_load_3d(&suf[0][0][0], &tm, tx * MIX_TS, ty * MIX_TS, 0, &bar);
  }
  if (!mbar_wait_bounded(&bar)) {
    atomicOr(d.err, EB_OUT_OF_RANGE);
    mbar_wait_bounded(&bar);  // second bounded wait for the copy in flight
    return;
  }
  // cell-centred fields for local cells -1..16 (2d/common/particle.f90:70-83), FP64 sums rounded to FP32
  for (int k = threadIdx.x; k < TT * TT; k += MP_THREADS) {
    const int r = k / TT + 1, c = k % TT + 1;  // staged node of local cell (c-2, r-2) ... origin at cell -2
    stmp[0][k] = make_float2((float)(0.5 * (suf[0][r][c] + suf[0][r + 1][c])),
                             (float)(0.5 * (suf[1][r][c] + suf[1][r][c + 1])));
    stmp[1][k] = make_float2((float)(0.25 * (suf[2][r][c] + suf[2][r][c + 1] + suf[2][r + 1][c] + suf[2][r + 1][c + 1])),
                             (float)(0.5 * (suf[3][r][c] + suf[3][r][c + 1])));
    stmp[2][k] = make_float2((float)(0.5 * (suf[4][r][c] + suf[4][r + 1][c])), (float)suf[5][r][c]);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < 2 * 3 * TW * JP; k += MP_THREADS) (&jhi[0][0][0])[k] = 0;
  __syncthreads();
  const float fs1 = m.fx_s1, fs2 = m.fx_s2, fis1 = 1.0f / m.fx_s1;

  const float dtdx = (float)(d.ph.delt * d.ph.d_delx);
  const float c = (float)d.ph.c;
  const float ic2 = (float)(1.0 / (d.ph.c * d.ph.c));
  const float third = 1.0f / 3.0f;
  const bool walls = d.ph.bc == BC_RECONNECTION;
  for (int isp = 0; isp < d.ph.nsp; ++isp) {
    const int bin = tile * d.ph.nsp + isp;
    const int n = m.cnt[bin];
    const size_t base = (size_t)bin * m.bcap;
    const float fac1 = (float)(d.ph.q[isp] / d.ph.r[isp] * 0.5 * d.ph.delt);
    const float txxx = fac1 * fac1;
    const float fac2 = (float)(d.ph.q[isp] * d.ph.delt / d.ph.r[isp]);
    const float qdd = (float)(d.ph.q[isp] * d.ph.delx * d.ph.d_delt);
    const float qs = (float)d.ph.q[isp];
    for (int s = threadIdx.x; s < n; s += MP_THREADS) {
      const size_t k = base + s;
      const int cl = m.P.cell[k];
      const int lx = cl & (MIX_TS - 1), ly = cl >> 4;
      const float ox = m.P.ox[k], oy = m.P.oy[k];
      float ux = m.P.ux[k], uy = m.P.uy[k], uz = m.P.uz[k];
      // quadratic spline weights at the old position, offsets -1, 0, +1
      const float sx0 = 0.5f * (1.f - ox) * (1.f - ox), sx1 = 0.75f - (ox - 0.5f) * (ox - 0.5f), sx2 = 0.5f * ox * ox;
      const float sy0 = 0.5f * (1.f - oy) * (1.f - oy), sy1 = 0.75f - (oy - 0.5f) * (oy - 0.5f), sy2 = 0.5f * oy * oy;
      float f[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int jy = 0; jy < 3; ++jy) {
        const float wy = jy == 0 ? sy0 : (jy == 1 ? sy1 : sy2);
        float fr[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int jx = 0; jx < 3; ++jx) {
          const float wx = jx == 0 ? sx0 : (jx == 1 ? sx1 : sx2);
          const int ci = (ly + jy) * TT + lx + jx;
          const float2 a = stmp[0][ci], b = stmp[1][ci], e = stmp[2][ci];
          fr[0] = fmaf(wx, a.x, fr[0]);
          fr[1] = fmaf(wx, a.y, fr[1]);
          fr[2] = fmaf(wx, b.x, fr[2]);
          fr[3] = fmaf(wx, b.y, fr[3]);
          fr[4] = fmaf(wx, e.x, fr[4]);
          fr[5] = fmaf(wx, e.y, fr[5]);
        }
#pragma unroll
        for (int q = 0; q < 6; ++q) f[q] = fmaf(wy, fr[q], f[q]);
      }
      const float bpx = f[0], bpy = f[1], bpz = f[2], epx = f[3], epy = f[4], epz = f[5];
      // Buneman-Boris (2d/common/particle.f90:133-155)
      float u1 = ux + fac1 * epx, u2 = uy + fac1 * epy, u3 = uz + fac1 * epz;
      const float g2 = c * c + u1 * u1 + u2 * u2 + u3 * u3;
      const float igam = rsqrtf(g2);
      const float gm = g2 * igam;
      const float fac1r = fac1 * igam;
      const float fac2r = __fdividef(fac2, gm + txxx * (bpx * bpx + bpy * bpy + bpz * bpz) * igam);
      const float u4 = u1 + fac1r * (u2 * bpz - u3 * bpy);
      const float u5 = u2 + fac1r * (u3 * bpx - u1 * bpz);
      const float u6 = u3 + fac1r * (u1 * bpy - u2 * bpx);
      u1 = u1 + fac2r * (u5 * bpz - u6 * bpy);
      u2 = u2 + fac2r * (u6 * bpx - u4 * bpz);
      u3 = u3 + fac2r * (u4 * bpy - u5 * bpx);
      ux = u1 + fac1 * epx;
      uy = u2 + fac1 * epy;
      uz = u3 + fac1 * epz;
      const float ig = rsqrtf(1.f + (ux * ux + uy * uy + uz * uz) * ic2);
      // move in cell units; integer cell + offset
      float nx_ = ox + ux * dtdx * ig, ny_ = oy + uy * dtdx * ig;
      float fx = floorf(nx_), fy = floorf(ny_);
      nx_ -= fx;
      ny_ -= fy;
      int incx = (int)fx, incy = (int)fy;
      if (nx_ >= 1.f) { nx_ = 0.f; incx += 1; }
      if (ny_ >= 1.f) { ny_ = 0.f; incy += 1; }
      if (walls) {
        // reflection about the walls at global cells 1 and nx-2 (nxs+1 and nxe-1 in reference indices),
        // all three momentum components reversed (2d/proj/reconnection/boundary_reconnection.f90:79-91)
        const int gxn = tx * MIX_TS + lx + incx;
        float X = (float)gxn + nx_;
        bool flip = false;
        if (gxn < 1) { X = 2.f - X; flip = true; }
        else if (gxn >= g.nx - 2) { X = 2.f * (float)(g.nx - 2) - X; flip = true; }
        if (flip) {
          ux = -ux; uy = -uy; uz = -uz;
          const float fX = floorf(X);
          nx_ = X - fX;
          incx = (int)fX - (tx * MIX_TS + lx);
          if (nx_ >= 1.f) { nx_ = 0.f; incx += 1; }
        }
      }
      if (incx < -1 || incx > 1 || incy < -1 || incy > 1) {
        atomicOr(d.err, EB_MOVED_TOO_FAR);
        incx = max(-1, min(1, incx));
        incy = max(-1, min(1, incy));
      }
      // ---- Esirkepov deposition on 4-wide windows (2d/common/field.f90:223-298) ----
      // window origin (node index space 0..4 = offsets -2..2): 0 if the particle moved to -1, else 1
      const int xa = incx < 0 ? 0 : 1, ya = incy < 0 ? 0 : 1;
      float s0x[4], s0y[4], dsx[4], dsy[4];
      s0x[0] = incx < 0 ? 0.f : sx0; s0x[1] = incx < 0 ? sx0 : sx1; s0x[2] = incx < 0 ? sx1 : sx2; s0x[3] = incx < 0 ? sx2 : 0.f;
      s0y[0] = incy < 0 ? 0.f : sy0; s0y[1] = incy < 0 ? sy0 : sy1; s0y[2] = incy < 0 ? sy1 : sy2; s0y[3] = incy < 0 ? sy2 : 0.f;
      shape_diff(ox, nx_, incx, dsx);
      shape_diff(oy, ny_, incy, dsy);
      const float gvz = uz * ig;
      const float qg = qs * gvz;
      float wy[4], wx[4], vy[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        wy[t] = -qdd * (s0y[t] + 0.5f * dsy[t]);
        wx[t] = -qdd * (s0x[t] + 0.5f * dsx[t]);
        vy[t] = qg * (0.5f * s0y[t] + third * dsy[t]);
      }
      const int nx0 = lx + xa, ny0 = ly + ya;  // sJ index of window node 0 (sJ origin = local cell -2)
      float px = 0.f, py = 0.f;
      const int b0 = ny0 * JP + nx0;  // word offset of window node (0, 0) in a plane
#pragma unroll
      for (int t = 0; t < 3; ++t) {
        px += dsx[t];
        py += dsy[t];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          const int ox_ = b0 + v * JP + t + 1, oy_ = b0 + (t + 1) * JP + v;
          fx_add(&jhi[0][0][0] + ox_, &jlo[0][0][0] + ox_, px * wy[v], fs1, fis1, fs2);
          fx_add(&jhi[1][0][0] + oy_, &jlo[1][0][0] + oy_, py * wx[v], fs1, fis1, fs2);
        }
      }
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const float zy = qg * (s0y[v] + 0.5f * dsy[v]);
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int oz_ = b0 + v * JP + t;
          fx_add(&jhi[2][0][0] + oz_, &jlo[2][0][0] + oz_, s0x[t] * zy + dsx[t] * vy[v], fs1, fis1, fs2);
        }
      }
      // ---- new cell, tile and bin code ----
      int nlx = lx + incx, nly = ly + incy;
      int ddx = nlx < 0 ? -1 : (nlx >= MIX_TS ? 1 : 0);
      int ddy = nly < 0 ? -1 : (nly >= MIX_TS ? 1 : 0);
      nlx -= ddx * MIX_TS;
      nly -= ddy * MIX_TS;
      int code = nly * MIX_TS + nlx;
      if (ddx != 0 || ddy != 0) code += ((ddy + 1) * 3 + (ddx + 1) + 1) * MIX_TC;
      m.P.cell[k] = code;
      m.P.ox[k] = nx_;
      m.P.oy[k] = ny_;
      m.P.ux[k] = ux;
      m.P.uy[k] = uy;
      m.P.uz[k] = uz;
    }
  }
  __syncthreads();
  // one flush of the tile into the global fixed-point current (exact 64-bit integer sums, so the
  // result does not depend on the order of the tiles); nodes wrap periodically in y, and in x
  // unless walls
  for (int k = threadIdx.x; k < 3 * TW * TW; k += MP_THREADS) {
    const int w = (k / TW) * JP + k % TW;
    const int ih = (&jhi[0][0][0])[w], il = (&jlo[0][0][0])[w];
    if ((ih | il) == 0) continue;
    const long long v = (long long)ih * 32768LL + (long long)il;
    const int comp = k / (TW * TW), r = (k / TW) % TW, cc = k % TW;
    int gx = tx * MIX_TS + cc - 2, gy = ty * MIX_TS + r - 2;
    if (gy < 0) gy += g.ny; else if (gy >= g.ny) gy -= g.ny;
    if (!walls) {
      if (gx < 0) gx += g.nx; else if (gx >= g.nx) gx -= g.nx;
    }
    atomicAdd(&m.ujx[(size_t)comp * g.fplane + (size_t)(gy + 2) * g.fp + gx + 2], (unsigned long long)v);
  }
}

void mix_push_deposit2d(const Dev2D& d, const void* tmap, cudaStream_t s) {
  cudaMemsetAsync(d.m.ujx, 0, sizeof(unsigned long long) * 3 * (size_t)d.g.fplane, s);
  k_mix_push<<<d.m.ntile, MP_THREADS, 0, s>>>(d, *(const CUtensorMap*)tmap);
}

// ghost refresh of uj after the flush (the fold is done by the index wrap above):
// rows nys-2, nys-1 <- nye-1, nye and nye+1, nye+2 <- nys, nys+1; columns likewise when periodic
__global__ void k_mix_refresh_y(Dev2D d) {
  const int ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= d.g.nx + 4) return;
  const size_t fp = d.g.fp;
  const int ny = d.g.ny;
  for (int k = 0; k < 3; ++k) {
    double* u = d.uj + (size_t)k * d.g.fplane + ii;
    u[(ny + 2) * fp] = u[2 * fp];
    u[(ny + 3) * fp] = u[3 * fp];
    u[0] = u[ny * fp];
    u[fp] = u[(ny + 1) * fp];
  }
}
__global__ void k_mix_refresh_x(Dev2D d) {
  const int jf = blockIdx.x * blockDim.x + threadIdx.x;
  if (jf >= d.g.ny + 4) return;
  const int nx = d.g.nx;
  for (int k = 0; k < 3; ++k) {
    double* u = d.uj + (size_t)k * d.g.fplane + (size_t)jf * d.g.fp;
    u[0] = u[nx];
    u[1] = u[nx + 1];
    u[nx + 2] = u[2];
    u[nx + 3] = u[3];
  }
}
// fixed point -> FP64 current over the whole ghosted extent
__global__ void k_mix_fix2d(Dev2D d) {
  const size_t n = (size_t)3 * d.g.fplane;
  const double is2 = d.m.fx_is2;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    d.uj[k] = (double)(long long)d.m.ujx[k] * is2;
}

void mix_curre_refresh2d(const Dev2D& d, cudaStream_t s) {
  k_mix_fix2d<<<4 * 152, 256, 0, s>>>(d);
  k_mix_refresh_y<<<(d.g.nx + 4 + 127) / 128, 128, 0, s>>>(d);
  if (d.ph.bc == BC_PERIODIC) k_mix_refresh_x<<<(d.g.ny + 4 + 127) / 128, 128, 0, s>>>(d);
}

// ---------------------------------------------------------------------------
// migration between bins.  Phase 1 (per bin): list the vacated slots in
// ascending order and copy the leavers, grouped by direction and in slot
// order, into the bin's leaver region.
// ---------------------------------------------------------------------------
constexpr int MG_THREADS = 256;
constexpr int MG_WARPS = MG_THREADS / 32;

__global__ void __launch_bounds__(MG_THREADS) k_mix_mig1(Dev2D d) {
  const Mix2D& m = d.m;
  const int bin = blockIdx.x;
  const int n = m.cnt[bin];
  const size_t base = (size_t)bin * m.bcap, lbase = (size_t)bin * m.lcap;
  // each warp owns a contiguous segment of the bin: count, then write in slot order
  __shared__ int wc[MG_WARPS][10];   // per warp: leavers per direction, [9] = all leavers
  __shared__ int wo[MG_WARPS][10];   // per warp: first output position per direction / hole list
  __shared__ int off9[9];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int seg = ((n + MG_WARPS - 1) / MG_WARPS + 31) & ~31;
  const int s_lo = min(n, warp * seg), s_hi = min(n, s_lo + seg);
  const unsigned lt = lanemask_lt();
  int cnt[10];
#pragma unroll
  for (int q = 0; q < 10; ++q) cnt[q] = 0;
  for (int s0 = s_lo; s0 < s_hi; s0 += 32) {
    const int s = s0 + lane;
    const int code = s < s_hi ? m.P.cell[base + s] : 0;
    const int q = code >= MIX_TC ? code / MIX_TC - 1 : -1;
    const unsigned any = __ballot_sync(0xffffffffu, q >= 0);
    if (!any) continue;
    cnt[9] += __popc(any);
#pragma unroll
    for (int dd = 0; dd < 9; ++dd) cnt[dd] += __popc(__ballot_sync(0xffffffffu, q == dd));
  }
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < 10; ++q) wc[warp][q] = cnt[q];
  }
  __syncthreads();
  if (threadIdx.x < 10) {
    const int q = threadIdx.x;
    int acc = 0;
    for (int w = 0; w < MG_WARPS; ++w) {
      wo[w][q] = acc;
      acc += wc[w][q];
    }
    if (q < 9) {
      m.lcnt[bin * 9 + q] = acc;
      off9[q] = acc;  // totals, turned into offsets below
    } else if (acc > m.lcap) {
      atomicOr(d.err, EB_CAPACITY);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int q = 0; q < 9; ++q) {
      const int t = off9[q];
      off9[q] = acc;
      m.lofs[bin * 9 + q] = acc;
      acc += t;
    }
  }
  __syncthreads();
  int run[10];
#pragma unroll
  for (int q = 0; q < 9; ++q) run[q] = off9[q] + wo[warp][q];
  run[9] = wo[warp][9];
  for (int s0 = s_lo; s0 < s_hi; s0 += 32) {
    const int s = s0 + lane;
    const int code = s < s_hi ? m.P.cell[base + s] : 0;
    const int q = code >= MIX_TC ? code / MIX_TC - 1 : -1;
    const unsigned any = __ballot_sync(0xffffffffu, q >= 0);
    if (!any) continue;
    int lpos = 0;
#pragma unroll
    for (int dd = 0; dd < 9; ++dd) {
      const unsigned b = __ballot_sync(0xffffffffu, q == dd);
      if (q == dd) lpos = run[dd] + __popc(b & lt);
      run[dd] += __popc(b);
    }
    const int hpos = run[9] + __popc(any & lt);
    run[9] += __popc(any);
    if (q >= 0 && lpos < m.lcap && hpos < m.lcap) {
      const size_t k = base + s, l = lbase + lpos;
      m.L.cell[l] = code % MIX_TC;
      m.L.ox[l] = m.P.ox[k];
      m.L.oy[l] = m.P.oy[k];
      m.L.ux[l] = m.P.ux[k];
      m.L.uy[l] = m.P.uy[k];
      m.L.uz[l] = m.P.uz[k];
      m.L.id[l] = m.P.id[k];
      m.holes[lbase + hpos] = s;
    }
  }
}

// Phase 2 (per bin): arrivals from the 8 neighbours, in direction order, fill the
// vacated slots in ascending order; extra arrivals are appended; if there are
// fewer arrivals than holes, the bin's tail (non-hole slots from the end
// downwards) fills the remaining holes below the new count.
__global__ void __launch_bounds__(MG_THREADS) k_mix_mig2(Dev2D d) {
  const Mix2D& m = d.m;
  const int bin = blockIdx.x;
  const int nsp = d.ph.nsp;
  const int tile = bin / nsp, isp = bin - tile * nsp;
  const int tx = tile % m.ntx, ty = tile / m.ntx;
  const size_t base = (size_t)bin * m.bcap, lbase = (size_t)bin * m.lcap;
  __shared__ int acnt[9], abase[9], asrc[9];
  __shared__ int sh_h, sh_b, sh_n;
  __shared__ int wcnt[MG_WARPS];
  __shared__ int tail_run;
  if (threadIdx.x < 9) {
    const int q = threadIdx.x;
    if (q == 4) {
      acnt[q] = 0;
      asrc[q] = bin;
    } else {
      int sx = tx - dir_dx(q), sy = ty - dir_dy(q);
      if (sx < 0) sx += m.ntx; else if (sx >= m.ntx) sx -= m.ntx;
      if (sy < 0) sy += m.nty; else if (sy >= m.nty) sy -= m.nty;
      const int sbin = (sy * m.ntx + sx) * nsp + isp;
      asrc[q] = sbin;
      acnt[q] = m.lcnt[sbin * 9 + q];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int q = 0; q < 9; ++q) {
      abase[q] = acc;
      acc += acnt[q];
    }
    int h = 0;
    for (int q = 0; q < 9; ++q) h += m.lcnt[bin * 9 + q];
    sh_h = h < m.lcap ? h : m.lcap;
    sh_b = acc;
    sh_n = m.cnt[bin];
    tail_run = 0;
  }
  __syncthreads();
  const int h = sh_h, b = sh_b, n = sh_n;
  int nn = n - h + b;
  if (nn > m.bcap) {
    if (threadIdx.x == 0) atomicOr(d.err, EB_CAPACITY);
    nn = m.bcap;
  }
  // tail stayers of [nn, n) in descending slot order
  if (b < h) {
    const unsigned lt = lanemask_lt();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t0 = n - 1; t0 >= nn; t0 -= MG_THREADS) {
      const int t = t0 - threadIdx.x;
      const bool st = t >= nn && m.P.cell[base + t] < MIX_TC;
      const unsigned bal = __ballot_sync(0xffffffffu, st);
      if (lane == 0) wcnt[warp] = __popc(bal);
      __syncthreads();
      int pos = tail_run;
      for (int w = 0; w < warp; ++w) pos += wcnt[w];
      if (st && pos + __popc(bal & lt) < m.lcap) m.tails[lbase + pos + __popc(bal & lt)] = t;
      __syncthreads();
      if (threadIdx.x == 0) {
        int add = 0;
        for (int w = 0; w < MG_WARPS; ++w) add += wcnt[w];
        tail_run += add;
      }
      __syncthreads();
    }
  }
  // fills: hole m <- arrival m (m < min(h, b)); slot n + (m - h) <- arrival m (h <= m < b);
  // hole m <- tail (m - b) for b <= m < h with holes[m] < nn
  const int total = b > h ? b : h;
  for (int q = threadIdx.x; q < total; q += MG_THREADS) {
    int dst = -1;
    bool from_arrival = q < b;
    if (q < h) {
      dst = m.holes[lbase + q];
      if (!from_arrival && dst >= nn) dst = -1;
    } else {
      dst = n + (q - h);
    }
    if (dst < 0 || dst >= m.bcap) continue;
    const size_t kd = base + dst;
    if (from_arrival) {
      int dq = 0;
      while (dq < 8 && q >= abase[dq + 1]) ++dq;
      const int sbin = asrc[dq];
      const int lpos = m.lofs[sbin * 9 + dq] + (q - abase[dq]);
      if (lpos >= m.lcap) continue;  // the source bin overflowed its leaver region (error already set)
      const size_t ks = (size_t)sbin * m.lcap + lpos;
      m.P.cell[kd] = m.L.cell[ks];
      m.P.ox[kd] = m.L.ox[ks];
      m.P.oy[kd] = m.L.oy[ks];
      m.P.ux[kd] = m.L.ux[ks];
      m.P.uy[kd] = m.L.uy[ks];
      m.P.uz[kd] = m.L.uz[ks];
      m.P.id[kd] = m.L.id[ks];
    } else {
      const size_t ks = base + m.tails[lbase + (q - b)];
      m.P.cell[kd] = m.P.cell[ks];
      m.P.ox[kd] = m.P.ox[ks];
      m.P.oy[kd] = m.P.oy[ks];
      m.P.ux[kd] = m.P.ux[ks];
      m.P.uy[kd] = m.P.uy[ks];
      m.P.uz[kd] = m.P.uz[ks];
      m.P.id[kd] = m.P.id[ks];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) m.cnt[bin] = nn;
}

void mix_migrate2d(const Dev2D& d, cudaStream_t s) {
  k_mix_mig1<<<d.m.nbin, MG_THREADS, 0, s>>>(d);
  k_mix_mig2<<<d.m.nbin, MG_THREADS, 0, s>>>(d);
}

// ---------------------------------------------------------------------------
// reference layout -> bins.  One CTA per bin of the staged tile rows; the
// particles of each cell come from the cell-sorted rows (cumcnt gives the
// ranges) and are dealt round-robin over the tile's cells.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(MIX_TC) k_mix_put(Dev2D d, const double* aos, int ndim, int np_host, int isp,
                                                   int ty0) {
  const Mix2D& m = d.m;
  const Grid2D g = d.g;
  const int tx = blockIdx.x, ty = ty0 + blockIdx.y;
  const int bin = (ty * m.ntx + tx) * d.ph.nsp + isp;
  const int lx = threadIdx.x & (MIX_TS - 1), ly = threadIdx.x >> 4;
  const int gx = tx * MIX_TS + lx, gy = ty * MIX_TS + ly;
  const int row = isp * g.ny + gy;
  const int* ccr = d.cc + (size_t)row * (g.nx + 1);
  const int first = ccr[gx];
  const int nmine = ccr[gx + 1] - first;
  __shared__ int wsum[MIX_TC / 32];
  __shared__ int sh_max, sh_base;
  if (threadIdx.x == 0) {
    sh_max = 0;
    sh_base = 0;
  }
  __syncthreads();
  atomicMax(&sh_max, nmine);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lt = lanemask_lt();
  // staged row (relative to this chunk): rows of species isp starting at tile row ty0
  const double* rowp = aos + (size_t)((ty - ty0) * MIX_TS + ly) * np_host * ndim;
  const double dxi = d.ph.d_delx;
  for (int k = 0; k < sh_max; ++k) {
    const bool has = k < nmine;
    const unsigned bal = __ballot_sync(0xffffffffu, has);
    if (lane == 0) wsum[warp] = __popc(bal);
    __syncthreads();
    int pos = sh_base;
    for (int w = 0; w < warp; ++w) pos += wsum[w];
    pos += __popc(bal & lt);
    if (has) {
      if (pos < m.bcap) {
        const double* a = rowp + (size_t)(first + k) * ndim;
        const size_t o = (size_t)bin * m.bcap + pos;
        m.P.cell[o] = ly * MIX_TS + lx;
        m.P.ox[o] = (float)(a[0] * dxi - (double)(g.nxgs + gx));
        m.P.oy[o] = (float)(a[1] * dxi - (double)(g.nygs + gy));
        m.P.ux[o] = (float)a[2];
        m.P.uy[o] = (float)a[3];
        m.P.uz[o] = (float)a[4];
        m.P.id[o] = ndim > 5 ? __double_as_longlong(a[5]) : 0;
      } else {
        atomicOr(d.err, EB_CAPACITY);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int add = 0;
      for (int w = 0; w < MIX_TC / 32; ++w) add += wsum[w];
      sh_base += add;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) m.cnt[bin] = sh_base < m.bcap ? sh_base : m.bcap;
}

void mix_put2d(const Dev2D& d, const double* aos, int ndim, int np_host, int isp, int ty0, int nty,
               cudaStream_t s) {
  dim3 grid(d.m.ntx, nty);
  k_mix_put<<<grid, MIX_TC, 0, s>>>(d, aos, ndim, np_host, isp, ty0);
}

// ---------------------------------------------------------------------------
// bins -> reference layout.  Per-cell counts (each cell belongs to one bin),
// per-row exclusive scan into cumcnt and np2, then one warp per bin writes its
// particles cell-sorted, keeping slot order inside a cell.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(MIX_TC) k_mix_cellcount(Dev2D d) {
  const Mix2D& m = d.m;
  const int bin = blockIdx.x;
  const int nsp = d.ph.nsp;
  const int tile = bin / nsp, isp = bin - tile * nsp;
  const int tx = tile % m.ntx, ty = tile / m.ntx;
  __shared__ int c[MIX_TC];
  c[threadIdx.x] = 0;
  __syncthreads();
  const int n = m.cnt[bin];
  for (int s = threadIdx.x; s < n; s += MIX_TC) atomicAdd(&c[m.P.cell[(size_t)bin * m.bcap + s] & (MIX_TC - 1)], 1);
  __syncthreads();
  const int lx = threadIdx.x & (MIX_TS - 1), ly = threadIdx.x >> 4;
  m.cellcnt[((size_t)isp * d.g.ny + ty * MIX_TS + ly) * d.g.nx + tx * MIX_TS + lx] = c[threadIdx.x];
}

__global__ void __launch_bounds__(32) k_mix_rowscan(Dev2D d) {
  const int row = blockIdx.x;
  const int lane = threadIdx.x;
  const int nx = d.g.nx;
  const int* cnt = d.m.cellcnt + (size_t)row * nx;
  int* ccr = d.cc + (size_t)row * (nx + 1);
  int carry = 0;
  for (int k0 = 0; k0 < nx; k0 += 32) {
    const int k = k0 + lane;
    const int v = k < nx ? cnt[k] : 0;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (k < nx) ccr[k] = incl - v + carry;
    carry += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (lane == 0) {
    ccr[nx] = carry;
    d.np2[row] = carry;
  }
}

void mix_count_rows2d(const Dev2D& d, cudaStream_t s) {
  k_mix_cellcount<<<d.m.nbin, MIX_TC, 0, s>>>(d);
  k_mix_rowscan<<<d.nrowjob, 32, 0, s>>>(d);
}

__global__ void __launch_bounds__(32) k_mix_get(Dev2D d, double* aos, int ndim, int np_host, int isp, int ty0) {
  const Mix2D& m = d.m;
  const Grid2D g = d.g;
  const int tx = blockIdx.x, ty = ty0 + blockIdx.y;
  const int bin = (ty * m.ntx + tx) * d.ph.nsp + isp;
  const int lane = threadIdx.x;
  __shared__ int off[MIX_TC];
  for (int c = lane; c < MIX_TC; c += 32) {
    const int gx = tx * MIX_TS + (c & (MIX_TS - 1)), gy = ty * MIX_TS + (c >> 4);
    off[c] = d.cc[((size_t)isp * g.ny + gy) * (g.nx + 1) + gx];
  }
  __syncwarp();
  const int n = m.cnt[bin];
  const unsigned lt = lanemask_lt();
  const double dx = d.ph.delx;
  for (int t0 = 0; t0 < n; t0 += 32) {
    const int t = t0 + lane;
    const bool act = t < n;
    const size_t k = (size_t)bin * m.bcap + t;
    const int c = act ? (m.P.cell[k] & (MIX_TC - 1)) : -1 - lane;
    const unsigned peers = __match_any_sync(0xffffffffu, c);
    int basepos = 0;
    if (act) basepos = off[c];
    __syncwarp();
    if (act && lane == __ffs(peers) - 1) off[c] = basepos + __popc(peers);
    __syncwarp();
    if (act) {
      const int pos = basepos + __popc(peers & lt);
      const int lx = c & (MIX_TS - 1), ly = c >> 4;
      const int gx = tx * MIX_TS + lx;
      if (pos < np_host) {
        double* a = aos + ((size_t)((ty - ty0) * MIX_TS + ly) * np_host + pos) * ndim;
        a[0] = ((double)(g.nxgs + gx) + (double)m.P.ox[k]) * dx;
        a[1] = ((double)(g.nygs + ty * MIX_TS + ly) + (double)m.P.oy[k]) * dx;
        a[2] = (double)m.P.ux[k];
        a[3] = (double)m.P.uy[k];
        a[4] = (double)m.P.uz[k];
        if (ndim > 5) a[5] = __longlong_as_double(m.P.id[k]);
      } else {
        atomicOr(d.err, EB_CAPACITY);
      }
    }
  }
}

void mix_get2d(const Dev2D& d, double* aos, int ndim, int np_host, int isp, int ty0, int nty, cudaStream_t s) {
  dim3 grid(d.m.ntx, nty);
  k_mix_get<<<grid, 32, 0, s>>>(d, aos, ndim, np_host, isp, ty0);
}

// ---------------------------------------------------------------------------
// device loader: the same plasma as load_weibel2d_ppc (same Philox counters:
// row-local particle index k = cx*ppc + kk, row jj), dealt into the bins
// round-robin over cells: slot s of a bin holds cell s % 256, copy s / 256.
// ---------------------------------------------------------------------------
__global__ void k_mix_load(Dev2D d, int ppc, unsigned long long seed, double drift, int axis, double u_thi,
                           double u_the) {
  const Mix2D& m = d.m;
  const Grid2D g = d.g;
  const int bin = blockIdx.y;
  const int nsp = d.ph.nsp;
  const int tile = bin / nsp, isp = bin - tile * nsp;
  const int tx = tile % m.ntx, ty = tile / m.ntx;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = MIX_TC * ppc;
  if (s == 0) m.cnt[bin] = n < m.bcap ? n : m.bcap;
  if (s >= n || s >= m.bcap) return;
  const int c = s % MIX_TC, kk = s / MIX_TC;
  const int lx = c & (MIX_TS - 1), ly = c >> 4;
  const int cx = tx * MIX_TS + lx, jj = ty * MIX_TS + ly;
  const int k = cx * ppc + kk;
  const uint2 key = make_uint2((unsigned)seed, (unsigned)(seed >> 32));
  const uint4 rp = philox4x32(make_uint4((unsigned)k, (unsigned)jj, 0u, 0u), key);
  const uint4 r1 = philox4x32(make_uint4((unsigned)k, (unsigned)jj, 1u + 2u * isp, 0u), key);
  const uint4 r2 = philox4x32(make_uint4((unsigned)k, (unsigned)jj, 2u + 2u * isp, 0u), key);
  const size_t o = (size_t)bin * m.bcap + s;
  m.P.cell[o] = c;
  float ox = (float)(1.0 - u01(rp.x, rp.y)), oy = (float)(1.0 - u01(rp.z, rp.w));
  if (ox >= 1.f) ox = 0.f;
  if (oy >= 1.f) oy = 0.f;
  m.P.ox[o] = ox;
  m.P.oy[o] = oy;
  const double sd = isp == 0 ? u_thi : u_the;
  const double twopi = 6.283185307179586;
  const double a1 = u01(r1.x, r1.y), b1 = u01(r1.z, r1.w), a2 = u01(r2.x, r2.y), b2 = u01(r2.z, r2.w);
  const double rad1 = sqrt(-2.0 * log(a1)), rad2 = sqrt(-2.0 * log(a2));
  double u[3] = {sd * rad1 * cos(twopi * b1), sd * rad1 * sin(twopi * b1), sd * rad2 * cos(twopi * b2)};
  if (isp == 1 && drift != 0.0) u[axis] += (k % 2 == 0) ? drift : -drift;
  m.P.ux[o] = (float)u[0];
  m.P.uy[o] = (float)u[1];
  m.P.uz[o] = (float)u[2];
  m.P.id[o] = -((long long)jj * g.nx * ppc + k + 1);
}

void mix_load_weibel2d(const Dev2D& d, int ppc, unsigned long long seed, double drift, int drift_axis,
                       double u_thi, double u_the, cudaStream_t s) {
  dim3 grid((MIX_TC * ppc + 255) / 256, d.m.nbin);
  k_mix_load<<<grid, 256, 0, s>>>(d, ppc, seed, drift, drift_axis, u_thi, u_the);
}

// kinetic energy sums in FP64 over the FP32 momenta (2d/proj/weibel/app.f90:507-519)
__global__ void __launch_bounds__(256) k_mix_energy(Dev2D d) {
  __shared__ double sh[256];
  const Mix2D& m = d.m;
  const int isp = blockIdx.y;
  const double c = d.ph.c, rr = d.ph.r[isp];
  double v = 0.0;
  for (int tile = blockIdx.x; tile < m.ntile; tile += gridDim.x) {
    const int bin = tile * d.ph.nsp + isp;
    const int n = m.cnt[bin];
    for (int s = threadIdx.x; s < n; s += 256) {
      const size_t k = (size_t)bin * m.bcap + s;
      const double a = m.P.ux[k], b = m.P.uy[k], e = m.P.uz[k];
      v += rr * (sqrt(1.0 + (a * a + b * b + e * e) / (c * c)) - 1.0);
    }
  }
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) d.partials[((size_t)isp * d.nred + blockIdx.x) * 2] = sh[0];
}

void mix_energy2d(const Dev2D& d, cudaStream_t s) {
  cudaMemsetAsync(d.partials, 0, sizeof(double) * 2 * 3 * (size_t)d.nred, s);
  const int nb = d.nred < d.m.ntile ? d.nred : d.m.ntile;
  k_mix_energy<<<dim3(nb, d.ph.nsp), 256, 0, s>>>(d);
  fast::energy_fields_fin2d(d, s);
}

}  // namespace wpic
