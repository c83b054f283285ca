// Mixed-precision 2D path: FP32 push, gather and deposition weights on
// integer-cell + FP32-offset positions; FP32 currents summed exactly in fixed
// point and converted to FP64 global J; FP64 field state and solver (the FP64
// kernels in fp2d.cuh).
//
// Storage: per (16 x 16-cell tile, species) bin, one column of slots per cell
// (slot (k, c) = k * 256 + c).  One CTA of 256 threads per tile runs
// particle__solv and ele_cur fused (2d/common/particle.f90:48-179,
// 2d/common/field.f90:189-316), thread c walking the column of cell c:
//  * the tile's E/B stencil (20 x 20 nodes x 6 components, FP64) arrives in
//    shared memory by one TMA tensor load and is averaged to cell centres in FP32;
//  * each particle is pushed in place;
//  * its Esirkepov current is added into the thread's registers, which hold
//    the cell's full 5 x 5 x 3 stencil (every particle of the column shares the
//    cell), and every MIX_FLUSH particles the registers are added into the tile's
//    fixed-point current in shared memory (exact integer atomics);
//  * the tile is added once into the global fixed-point current.
// The periodic wraps of boundary_periodic__particle_x/_y are integer cell
// arithmetic here; the conducting-wall reflection of
// boundary_reconnection__particle_x is applied before the deposit, as in the
// reconnection driver's order.  Particles that changed cell then move between
// columns by a deterministic two-kernel migration: each column's holes are
// filled in slot order from its arrivals (neighbour cells in direction order),
// extra arrivals appended, and with fewer arrivals than holes the column's tail
// fills the remaining holes -- the reference's row scheme
// (2d/common/boundary_periodic.f90:193-225) applied to a cell column.
#include <cuda.h>

#include <cmath>

#include "common.cuh"
#include "mixed_common.cuh"

namespace wpic {

namespace {

constexpr int MP_THREADS = MIX_TC;  // one thread per cell of the tile
constexpr int TW = MIX_TS + 4;      // staged field nodes per tile edge (cells -2 .. 17)
constexpr int TT = MIX_TS + 2;      // cell-centred values per tile edge (cells -1 .. 16)
constexpr int FLUSH_EVERY = MIX_FLUSH;  // particles accumulated in registers between flushes
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

// 16-byte asynchronous global -> shared copy (both addresses 16-byte aligned)
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Mirror image X' = 2 W - X of the position X = cell + off about W = wc + wf (wf in [0, 1)), in
// split form: the integer parts cancel exactly and only the fractions are rounded.
__device__ __forceinline__ void reflect_split(int& cell, float& off, int wc, float wf) {
  const float r = (wf - off) + wf;  // in (-1, 2)
  const float fr = floorf(r);
  cell = 2 * wc - cell + (int)fr;
  off = r - fr;
  if (off >= 1.f) { off = 0.f; cell += 1; }
}

// direction code d = (dy + 1) * 3 + (dx + 1) of a move (4 = same cell) -> group index 0..7
__device__ __forceinline__ int dir_group(int d) { return d < 4 ? d : d - 1; }

// a0 += x0 y0, a1 += x1 y1 as one packed FP32x2 fused multiply-add (each lane rounds as fmaf)
__device__ __forceinline__ void ffma2_into(float& a0, float& a1, float x0, float x1, float y0, float y1) {
  const float2 r = __ffma2_rn(make_float2(x0, x1), make_float2(y0, y1), make_float2(a0, a1));
  a0 = r.x;
  a1 = r.y;
}

}  // namespace

// ---------------------------------------------------------------------------
// The push with the register current for the particles that stay in their cell only:
// a stayer's Esirkepov support is its cell's 3 x 3 nodes, so 21 registers
// hold it (2 x 3 x-edges, 3 x 2 y-edges, 3 x 3 z-nodes); a particle that changes cell (4 in 100
// per step on the 2D Weibel workload) joins its warp's queue, and 32 of them at a time, one lane each, claim their
// arrival slots, are deposited straight into the tile's fixed-point current and are written to
// their new columns.  With the smaller stencil and shared memory laid out for it (the TMA
// staging area becomes the queues and the per-thread staging slots once the cell-centred fields
// exist), three CTAs of 256 threads share an SM.
// ---------------------------------------------------------------------------
constexpr int PF2 = 3;  // particles in flight per thread (as fast as four; the fourth slot's 8 KB holds the queues)
constexpr int LQ2 = 64;                          // leaver queue entries per warp
constexpr int LQ2V = 3;                          // float4 per entry: (ox, oy, q vz, packed (inc, species, cell)),
                                                 // then the new slot's two float4
constexpr int LQ2_BYTES = (MP_THREADS / 32) * LQ2V * LQ2 * 16;
constexpr int PEND2_BYTES = 8 * MP_THREADS * 4;  // per thread: a leaver's new slot, staged until its queue index is known
constexpr int STAGE2_BYTES = 6 * TW * TW * 8;
constexpr int A2_BYTES = (STAGE2_BYTES > LQ2_BYTES + PEND2_BYTES ? STAGE2_BYTES : LQ2_BYTES + PEND2_BYTES);
constexpr int OFF2_J = (A2_BYTES + 127) / 128 * 128;
constexpr int OFF2_SFA = OFF2_J + 2 * 3 * TW * TW * 4;
constexpr int OFF2_SFB = OFF2_SFA + TT * TT * 16;
constexpr int OFF2_RING = OFF2_SFB + TT * TT * 8;
constexpr int PUSH2_SMEM = OFF2_RING + PF2 * MIX_W * MIX_TC * 4;
static_assert(OFF2_SFA % 16 == 0 && OFF2_RING % 16 == 0, "shared-memory alignment");
// three CTAs per SM: 228 KB of shared memory per SM, 1 KB of it reserved per CTA, and the
// kernel's static shared memory (under 512 bytes)
static_assert(3 * (PUSH2_SMEM + 512 + 1024) <= 228 * 1024, "three CTAs of k_mix_push2 per SM");

// Esirkepov current of one cell-leaver on the 5 x 5 stencil of its old cell (lx, ly), each value
// added to the tile's fixed-point planes (pitch TW); the same arithmetic as the register path.
// The three components are formed one after the other so that few weights are live at once
// (the queue drain runs inside the particle loop, beside the register current).
__device__ __forceinline__ void deposit_leaver2(float ox, float oy, float px_, float py_, int incx, int incy,
                                                int lx, int ly, float qdd, float qg, int* jhi, int* jlo, float s1,
                                                float is1, float s2) {
  const float third = 1.0f / 3.0f;
  float dsx[5], dsy[5];
  shape_diff5(ox, px_, incx, dsx);
  shape_diff5(oy, py_, incy, dsy);
  const float sx0 = 0.5f * (1.f - ox) * (1.f - ox), sx1 = 0.75f - (ox - 0.5f) * (ox - 0.5f), sx2 = 0.5f * ox * ox;
  const float sy0 = 0.5f * (1.f - oy) * (1.f - oy), sy1 = 0.75f - (oy - 0.5f) * (oy - 0.5f), sy2 = 0.5f * oy * oy;
  const float s0x[5] = {0.f, sx0, sx1, sx2, 0.f};
  const float s0y[5] = {0.f, sy0, sy1, sy2, 0.f};
  const float hq = -0.5f * qdd;
  {  // jx on the x-edges (kk + 1, e)
    float w[5];
#pragma unroll
    for (int e = 0; e < 5; ++e) w[e] = (e == 0 || e == 4) ? hq * dsy[e] : -qdd * (s0y[e] + 0.5f * dsy[e]);
    float px = 0.f;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      px += dsx[kk];
#pragma unroll
      for (int e = 0; e < 5; ++e) {
        const float v = px * w[e];
        if (v != 0.f) {
          const int a = (0 * TW + ly + e) * TW + lx + kk + 1;
          fx_add(jhi + a, jlo + a, v, s1, is1, s2);
        }
      }
    }
  }
  {  // jy on the y-edges (e, kk + 1)
    float w[5];
#pragma unroll
    for (int e = 0; e < 5; ++e) w[e] = (e == 0 || e == 4) ? hq * dsx[e] : -qdd * (s0x[e] + 0.5f * dsx[e]);
    float py = 0.f;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      py += dsy[kk];
#pragma unroll
      for (int e = 0; e < 5; ++e) {
        const float v = py * w[e];
        if (v != 0.f) {
          const int a = (1 * TW + ly + kk + 1) * TW + lx + e;
          fx_add(jhi + a, jlo + a, v, s1, is1, s2);
        }
      }
    }
  }
  // jz on the nodes (i, j)
  const float hg = 0.5f * qg, tg = third * qg;
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    const float zy = (j == 0 || j == 4) ? hg * dsy[j] : qg * (s0y[j] + 0.5f * dsy[j]);
    const float vy = (j == 0 || j == 4) ? tg * dsy[j] : qg * (0.5f * s0y[j] + third * dsy[j]);
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      const float v = dsx[i] * vy + s0x[i] * zy;
      if (v != 0.f) {
        const int a = (2 * TW + ly + j) * TW + lx + i;
        fx_add(jhi + a, jlo + a, v, s1, is1, s2);
      }
    }
  }
}

struct StayCurrent {
  float jx[2][3], jy[2][3], jz[3][3];
};

__device__ __forceinline__ void stay_zero(StayCurrent& a) {
#pragma unroll
  for (int k = 0; k < 2; ++k)
#pragma unroll
    for (int e = 0; e < 3; ++e) a.jx[k][e] = a.jy[k][e] = 0.f;
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i) a.jz[j][i] = 0.f;
}

// x-edge (k, e) of the register stencil at patch node (lx + k + 2, ly + e + 1); y-edge (k, e) at
// (lx + e + 1, ly + k + 2); z (j, i) at (lx + i + 1, ly + j + 1)
__device__ __forceinline__ void stay_flush(StayCurrent& a, int* jhi, int* jlo, int lx, int ly, float s1, float is1,
                                           float s2) {
#pragma unroll
  for (int k = 0; k < 2; ++k)
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      const int wx = (0 * TW + ly + e + 1) * TW + lx + k + 2;
      const int wy = (1 * TW + ly + k + 2) * TW + lx + e + 1;
      fx_add(jhi + wx, jlo + wx, a.jx[k][e], s1, is1, s2);
      fx_add(jhi + wy, jlo + wy, a.jy[k][e], s1, is1, s2);
    }
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const int w = (2 * TW + ly + j + 1) * TW + lx + i + 1;
      fx_add(jhi + w, jlo + w, a.jz[j][i], s1, is1, s2);
    }
  stay_zero(a);
}

// WALLS: the reconnection or shock boundary in x (false: periodic, the boundary code left out of
// the particle loop)
template <bool VAY, bool WALLS>
__global__ void __launch_bounds__(MP_THREADS, 3) k_mix_push2(Dev2D d, const __grid_constant__ CUtensorMap tm) {
  extern __shared__ __align__(128) unsigned char smem2[];
  double(*suf)[TW][TW] = reinterpret_cast<double(*)[TW][TW]>(smem2);
  float4* const lqueue = reinterpret_cast<float4*>(smem2);             // [warp][LQ2V][LQ2], after staging
  float4* const pend4 = reinterpret_cast<float4*>(smem2 + LQ2_BYTES);  // [256][2], after staging
  int* const jhi = reinterpret_cast<int*>(smem2 + OFF2_J);             // [3][TW][TW]
  int* const jlo = jhi + 3 * TW * TW;
  float4* const sfa = reinterpret_cast<float4*>(smem2 + OFF2_SFA);     // (Bx, By, Bz, Ex) at cell centres
  float2* const sfb = reinterpret_cast<float2*>(smem2 + OFF2_SFB);     // (Ey, Ez)
  float4* const ring = reinterpret_cast<float4*>(smem2 + OFF2_RING);   // [PF2][256] slots of 2 float4
  __shared__ __align__(8) unsigned long long bar;
  __shared__ int nb_bin[2][9], nb_dep[2][9];
  __shared__ long long nb_off[2][9];
  const Mix2D& m = d.m;
  const int tile = blockIdx.x;
  const int tx = tile % m.ntx, ty = tile / m.ntx;
  const Grid2D g = d.g;
  const int c = threadIdx.x;
  const int lane = c & 31;
  const int nsp = d.ph.nsp;
  const int bin0 = tile * nsp;
  const int n0 = m.cnt[bin0 * MIX_TC + c];
  const int ntot = n0 + (nsp > 1 ? m.cnt[(bin0 + 1) * MIX_TC + c] : 0);
  if (c < 2 * 9) {
    const int s = c / 9, q = c % 9;
    int ntx_ = tx + q % 3 - 1, nty_ = ty + q / 3 - 1;
    if (ntx_ < 0) ntx_ += m.ntx; else if (ntx_ >= m.ntx) ntx_ -= m.ntx;
    if (nty_ < 0) nty_ += m.nty; else if (nty_ >= m.nty) nty_ -= m.nty;
    const int b = (nty_ * m.ntx + ntx_) * nsp + (s < nsp ? s : 0);
    nb_bin[s][q] = b;
    nb_dep[s][q] = m.bdep[b];
    nb_off[s][q] = m.boff[b];
  }
  float* const col0 = mix_slot(m, bin0, 0, c);
  float* const col1 = mix_slot(m, bin0 + (nsp > 1 ? 1 : 0), 0, c) - (size_t)n0 * MIX_PL;
  // particle t goes to ring slot t mod PF2 (rs, kept by the loop)
  auto issue = [&](int t, int rs) {
    if (t < ntot) {
      const float* src = (t < n0 ? col0 : col1) + (size_t)t * MIX_PL;
      float4* dst = ring + (rs * MIX_TC + c) * 2;
      cp_async16(dst, src);
      cp_async16(dst + 1, src + 4);
    }
    cp_async_commit();
  };
#pragma unroll
  for (int t = 0; t < PF2; ++t) issue(t, t);
  if (c == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (c == 0) {
    mbar_expect_tx(&bar, (unsigned)STAGE2_BYTES);
    tma_load_3d(&suf[0][0][0], &tm, tx * MIX_TS, ty * MIX_TS, 0, &bar);
  }
  // every thread waits (bounded) for the tile; the CTA gives up together if any wait ran out
  const bool staged = mbar_wait_bounded(&bar);
  if (!__syncthreads_and(staged)) {
    if (c == 0) atomicOr(d.err, EB_STAGING_TIMEOUT);
    if (!staged) mbar_wait_bounded(&bar);
    cp_async_wait<0>();
    return;
  }
  for (int k = c; k < TT * TT; k += MP_THREADS) {
    const int r = k / TT + 1, cc = k % TT + 1;
    sfa[k] = make_float4((float)(0.5 * (suf[0][r][cc] + suf[0][r + 1][cc])),
                         (float)(0.5 * (suf[1][r][cc] + suf[1][r][cc + 1])),
                         (float)(0.25 * (suf[2][r][cc] + suf[2][r][cc + 1] + suf[2][r + 1][cc] + suf[2][r + 1][cc + 1])),
                         (float)(0.5 * (suf[3][r][cc] + suf[3][r][cc + 1])));
    sfb[k] = make_float2((float)(0.5 * (suf[4][r][cc] + suf[4][r + 1][cc])), (float)suf[5][r][cc]);
  }
  for (int k = c; k < 2 * 3 * TW * TW; k += MP_THREADS) jhi[k] = 0;
  __syncthreads();  // the staging area is free from here on (queue and pending leavers)
  const float fs1 = m.fx_s1, fs2 = m.fx_s2, fis1 = m.fx_is1f;
  const int lx = c & (MIX_TS - 1), ly = c >> 4;
  const float dtdx = m.k_dtdx;
  const float cl = m.k_c;
  const float ic2 = m.k_ic2;
  const float third = 1.0f / 3.0f;
  constexpr bool walls = WALLS;
  const int f0 = ly * TT + lx;
  StayCurrent acc;
  stay_zero(acc);
  float4* const myq = lqueue + (c >> 5) * LQ2V * LQ2;
  int qhead = 0, qtail = 0;  // the warp's leaver queue (warp-uniform)
  // 32 leavers at a time, one per lane: claim the arrival slot (arrival number pos goes to slot
  // depth - 1 - pos of the new column), deposit the current while the atomic is in flight, then
  // write the slot (its key word holds the direction group and the index in the old column)
  auto drain = [&](int cnt) {
    if (lane < cnt) {
      const int e = (qhead + lane) & (LQ2 - 1);
      const float4 a = myq[e];
      const int pk = __float_as_int(a.w);
      const int incx = (pk & 3) - 1, incy = ((pk >> 2) & 3) - 1, s = (pk >> 4) & 1, cc = pk >> 8;
      const int olx = cc & (MIX_TS - 1), oly = cc >> 4;
      const int nlx = olx + incx, nly = oly + incy;
      const int q = ((nly >> 4) + 1) * 3 + ((nlx >> 4) + 1);
      const int dlc = (nly & (MIX_TS - 1)) * MIX_TS + (nlx & (MIX_TS - 1));
      const int pos = atomicAdd(&m.acnt[nb_bin[s][q] * MIX_TC + dlc], 1);
      {
        const float4 b = myq[LQ2 + e];
        deposit_leaver2(a.x, a.y, b.x, b.y, incx, incy, olx, oly, s ? m.k_qdd[1] : m.k_qdd[0], a.z, jhi, jlo, fs1,
                        fis1, fs2);
      }
      const int dep = nb_dep[s][q];
      if (pos >= dep) {
        atomicOr(d.err, EB_CAPACITY);
      } else {
        float4* io = reinterpret_cast<float4*>(m.P + (((size_t)nb_off[s][q] + dep - 1 - pos) * MIX_TC + dlc) * MIX_W);
        io[0] = myq[LQ2 + e];
        io[1] = myq[2 * LQ2 + e];
      }
    }
    qhead += cnt;
    __syncwarp();
  };
  int j0 = 0, j1 = 0;
  int tw = ntot;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) tw = max(tw, __shfl_xor_sync(0xffffffffu, tw, o));
  int rs = 0;
  for (int t = 0; t < tw; ++t) {
    cp_async_wait<PF2 - 1>();
    bool leaves = false;
    float lq0 = 0.f, lq1 = 0.f, lq2 = 0.f;
    int lpk = 0;
    if (t < ntot) {
      const bool sp1 = t >= n0;
      const int k = sp1 ? t - n0 : t;
      const float4 pa = ring[(rs * MIX_TC + c) * 2], pb = ring[(rs * MIX_TC + c) * 2 + 1];
      const float ox = pa.x, oy = pa.y;
      float ux = pa.z, uy = pa.w, uz = pb.x;
      const float idlo = pb.y, idhi = pb.z;
      const float fac1 = sp1 ? m.k_fac1[1] : m.k_fac1[0];
      const float fac2 = sp1 ? m.k_fac2[1] : m.k_fac2[0];
      const float qdd = sp1 ? m.k_qdd[1] : m.k_qdd[0];
      const float qs = sp1 ? m.k_q[1] : m.k_q[0];
      const float txxx = fac1 * fac1;
      const float sx0 = 0.5f * (1.f - ox) * (1.f - ox), sx1 = 0.75f - (ox - 0.5f) * (ox - 0.5f), sx2 = 0.5f * ox * ox;
      const float sy0 = 0.5f * (1.f - oy) * (1.f - oy), sy1 = 0.75f - (oy - 0.5f) * (oy - 0.5f), sy2 = 0.5f * oy * oy;
      float f[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int jy = 0; jy < 3; ++jy) {
        const float wy = jy == 0 ? sy0 : (jy == 1 ? sy1 : sy2);
#pragma unroll
        for (int jx = 0; jx < 3; ++jx) {
          const float w = wy * (jx == 0 ? sx0 : (jx == 1 ? sx1 : sx2));
          const float4 a = sfa[f0 + jy * TT + jx];
          const float2 b = sfb[f0 + jy * TT + jx];
          ffma2_into(f[0], f[1], w, w, a.x, a.y);
          ffma2_into(f[2], f[3], w, w, a.z, a.w);
          ffma2_into(f[4], f[5], w, w, b.x, b.y);
        }
      }
      const float bpx = f[0], bpy = f[1], bpz = f[2], epx = f[3], epy = f[4], epz = f[5];
      float ig;
      if constexpr (VAY) {
        const float fac1r = fac1 * rsqrtf(cl * cl + ux * ux + uy * uy + uz * uz);
        const float u4 = ux + fac2 * epx + fac1r * (uy * bpz - uz * bpy);
        const float u5 = uy + fac2 * epy + fac1r * (uz * bpx - ux * bpz);
        const float u6 = uz + fac2 * epz + fac1r * (ux * bpy - uy * bpx);
        const float icl = ic2 * cl;
        const float tx_ = fac1 * bpx * icl, ty_ = fac1 * bpy * icl, tz_ = fac1 * bpz * icl;
        const float tau2 = tx_ * tx_ + ty_ * ty_ + tz_ * tz_;
        const float ua = (u4 * tx_ + u5 * ty_ + u6 * tz_) * icl;
        const float sigma = 1.f + (u4 * u4 + u5 * u5 + u6 * u6) * ic2 - tau2;
        const float gam2 = 0.5f * (sigma + sqrtf(sigma * sigma + 4.f * (tau2 + ua * ua)));
        ig = rsqrtf(gam2);
        const float gv = gam2 * ig;
        const float tt = __fdividef(1.f, tau2 + gam2);
        ux = tt * (gam2 * u4 + cl * ua * tx_ + gv * (u5 * tz_ - u6 * ty_));
        uy = tt * (gam2 * u5 + cl * ua * ty_ + gv * (u6 * tx_ - u4 * tz_));
        uz = tt * (gam2 * u6 + cl * ua * tz_ + gv * (u4 * ty_ - u5 * tx_));
      } else {
        float u1 = ux + fac1 * epx, u2 = uy + fac1 * epy, u3 = uz + fac1 * epz;
        const float g2 = cl * cl + u1 * u1 + u2 * u2 + u3 * u3;
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
        ig = rsqrtf(1.f + (ux * ux + uy * uy + uz * uz) * ic2);
      }
      float nx_ = ox + ux * dtdx * ig, ny_ = oy + uy * dtdx * ig;
      int incx = 0, incy = 0;
      if (nx_ >= 1.f) { nx_ -= 1.f; incx = 1; } else if (nx_ < 0.f) { nx_ += 1.f; incx = -1; }
      if (ny_ >= 1.f) { ny_ -= 1.f; incy = 1; } else if (ny_ < 0.f) { ny_ += 1.f; incy = -1; }
      if (nx_ >= 1.f) { nx_ = 0.f; incx += 1; }
      if (ny_ >= 1.f) { ny_ = 0.f; incy += 1; }
      if (nx_ < 0.f || nx_ >= 1.f || ny_ < 0.f || ny_ >= 1.f) {
        atomicOr(d.err, EB_MOVED_TOO_FAR);
        nx_ = fminf(fmaxf(nx_, 0.f), 0.99999994f);
        ny_ = fminf(fmaxf(ny_, 0.f), 0.99999994f);
      }
      if (walls) {
        const int gx0 = tx * MIX_TS + lx;
        int gxn = gx0 + incx;
        const bool shock = d.ph.bc == BC_SHOCK;
        const int lo_wall = shock ? g.wx0 + 1 : 1;
        bool flip = false;
        if (gxn < lo_wall) {
          reflect_split(gxn, nx_, lo_wall, 0.f);
          ux = -ux;
          flip = true;
        } else if (shock ? (gxn > m.k_xend_cell || (gxn == m.k_xend_cell && nx_ > m.k_xend_frac)) : gxn >= g.nx - 2) {
          if (shock) reflect_split(gxn, nx_, m.k_xend_cell, m.k_xend_frac);
          else reflect_split(gxn, nx_, g.nx - 2, 0.f);
          ux = shock ? 2.f * m.k_u0 - ux : -ux;
          flip = true;
        }
        if (flip) {
          uy = -uy; uz = -uz;
          incx = gxn - gx0;
          if (incx < -1 || incx > 1) {
            atomicOr(d.err, EB_MOVED_TOO_FAR);
            incx = max(-1, min(1, incx));
          }
        }
      }
      const float qg = qs * uz * ig;  // q * vz
      leaves = (incx | incy) != 0;
      if (leaves) {
        pend4[2 * c] = make_float4(nx_, ny_, ux, uy);
        pend4[2 * c + 1] = make_float4(uz, idlo, idhi, __int_as_float((dir_group((incy + 1) * 3 + (incx + 1)) << 16) | k));
        lq0 = ox; lq1 = oy; lq2 = qg;
        lpk = (incx + 1) | ((incy + 1) << 2) | ((sp1 ? 1 : 0) << 4) | (c << 8);
      } else {
        float4* so = reinterpret_cast<float4*>((sp1 ? col1 + (size_t)n0 * MIX_PL : col0) +
                                               (size_t)(sp1 ? j1 : j0) * MIX_PL);
        so[0] = make_float4(nx_, ny_, ux, uy);
        so[1] = make_float4(uz, idlo, idhi, 0.f);  // a stayer's key word is not read
        if (sp1) ++j1; else ++j0;
        // Esirkepov on the cell's 3 x 3 nodes: the factored spline differences of a move inside
        // the cell (2d/common/field.f90:223-298)
        const float dlx = nx_ - ox, spx = ox + nx_, dly = ny_ - oy, spy = oy + ny_;
        const float dsx[3] = {-0.5f * dlx * (2.f - spx), -dlx * (spx - 1.f), 0.5f * dlx * spx};
        const float dsy[3] = {-0.5f * dly * (2.f - spy), -dly * (spy - 1.f), 0.5f * dly * spy};
        const float s0x[3] = {sx0, sx1, sx2}, s0y[3] = {sy0, sy1, sy2};
        const float px[2] = {dsx[0], dsx[0] + dsx[1]}, py[2] = {dsy[0], dsy[0] + dsy[1]};
        float wyq[3], wxq[3], zy[3], vy[3];
#pragma unroll
        for (int e = 0; e < 3; ++e) {
          wyq[e] = -qdd * (s0y[e] + 0.5f * dsy[e]);
          wxq[e] = -qdd * (s0x[e] + 0.5f * dsx[e]);
          zy[e] = qg * (s0y[e] + 0.5f * dsy[e]);
          vy[e] = qg * (0.5f * s0y[e] + third * dsy[e]);
        }
#pragma unroll
        for (int kk = 0; kk < 2; ++kk)
#pragma unroll
          for (int e = 0; e < 3; ++e) {
            acc.jx[kk][e] = fmaf(px[kk], wyq[e], acc.jx[kk][e]);
            acc.jy[kk][e] = fmaf(py[kk], wxq[e], acc.jy[kk][e]);
          }
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          ffma2_into(acc.jz[j][0], acc.jz[j][1], dsx[0], dsx[1], vy[j], vy[j]);
          acc.jz[j][2] = fmaf(dsx[2], vy[j], acc.jz[j][2]);
          ffma2_into(acc.jz[j][0], acc.jz[j][1], s0x[0], s0x[1], zy[j], zy[j]);
          acc.jz[j][2] = fmaf(s0x[2], zy[j], acc.jz[j][2]);
        }
      }
    }
    // leavers join the warp's queue; with 32 waiting they are deposited and written one per lane
    const unsigned lm = __ballot_sync(0xffffffffu, leaves);
    if (leaves) {
      const int e = (qtail + __popc(lm & ((1u << lane) - 1u))) & (LQ2 - 1);
      myq[e] = make_float4(lq0, lq1, lq2, __int_as_float(lpk));
      myq[LQ2 + e] = pend4[2 * c];
      myq[2 * LQ2 + e] = pend4[2 * c + 1];
    }
    qtail += __popc(lm);
    __syncwarp();
    if (qtail - qhead >= 32) drain(32);
    if ((t & (FLUSH_EVERY - 1)) == FLUSH_EVERY - 1) stay_flush(acc, jhi, jlo, lx, ly, fs1, fis1, fs2);
    issue(t + PF2, rs);
    rs = rs == PF2 - 1 ? 0 : rs + 1;
  }
  cp_async_wait<0>();
  if (qtail > qhead) drain(qtail - qhead);
  m.ccnt[bin0 * MIX_TC + c] = j0;
  if (nsp > 1) m.ccnt[(bin0 + 1) * MIX_TC + c] = j1;
  if (tw & (FLUSH_EVERY - 1)) stay_flush(acc, jhi, jlo, lx, ly, fs1, fis1, fs2);
  __syncthreads();
  for (int k = c; k < 3 * TW * TW; k += MP_THREADS) {
    const int ih = jhi[k], il = jlo[k];
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

void mix_push_deposit2d(const Dev2D& d, const void* tmap, bool vay, cudaStream_t s) {
  cudaMemsetAsync(d.m.ujx, 0, sizeof(unsigned long long) * 3 * (size_t)d.g.fplane, s);
  const CUtensorMap& tm = *(const CUtensorMap*)tmap;
  const bool walls = d.ph.bc != BC_PERIODIC;
  if (vay && walls) k_mix_push2<true, true><<<d.m.ntile, MP_THREADS, PUSH2_SMEM, s>>>(d, tm);
  else if (vay) k_mix_push2<true, false><<<d.m.ntile, MP_THREADS, PUSH2_SMEM, s>>>(d, tm);
  else if (walls) k_mix_push2<false, true><<<d.m.ntile, MP_THREADS, PUSH2_SMEM, s>>>(d, tm);
  else k_mix_push2<false, false><<<d.m.ntile, MP_THREADS, PUSH2_SMEM, s>>>(d, tm);
}

// fixed point -> FP64 current over the whole ghosted extent
__global__ void k_mix_fix2d(Dev2D d) {
  const size_t n = (size_t)3 * d.g.fplane;
  const double is2 = d.m.fx_is2;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    d.uj[k] = (double)(long long)d.m.ujx[k] * is2;
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

void mix_curre_refresh2d(const Dev2D& d, cudaStream_t s) {
  k_mix_fix2d<<<4 * 152, 256, 0, s>>>(d);
  k_mix_refresh_y<<<(d.g.nx + 4 + 127) / 128, 128, 0, s>>>(d);
  if (d.ph.bc == BC_PERIODIC) k_mix_refresh_x<<<(d.g.ny + 4 + 127) / 128, 128, 0, s>>>(d);
}

// ---------------------------------------------------------------------------
// arrivals (per bin, thread = destination cell): the push left the cell's j stayers in slots
// 0 .. j-1 and its b arrivals in slots dep-1 down to dep-b, in the order the push's atomics
// handed out.  They are moved to slots j .. j+b-1 in the order of their keys -- direction
// group, then slot in the source column -- so the result does not depend on that order.
// This keeps the reference's scheme of arrivals taking the free slots of a row
// (2d/common/boundary_periodic.f90:193-225), applied to a cell column.  The kernel also
// records, per bin, count + 2 x arrivals of its fullest column, the room the next step may
// need; past 7/8 of the depth the host grows the bin before the next push.
// ---------------------------------------------------------------------------
constexpr int ARR_KR = 8;     // keys per cell held in registers; more are read from global memory
constexpr int ARR_BATCH = 4;

__global__ void __launch_bounds__(MIX_TC) k_mix_arrive(Dev2D d) {
  __shared__ int wmax[MIX_TC / 32];
  const Mix2D& m = d.m;
  const int bin = blockIdx.x;
  const int c = threadIdx.x;
  const int dep = m.bdep[bin];
  const int nold = m.cnt[bin * MIX_TC + c];
  const int j = m.ccnt[bin * MIX_TC + c];
  int b = m.acnt[bin * MIX_TC + c];
  bool ok = true;
  // the arrivals must not have reached the slots the push read (nold) or the moved arrivals' range
  if (b > dep || nold + b > dep || j + 2 * b > dep) {
    ok = false;
    atomicOr(d.err, EB_CAPACITY);
  }
  if (b > dep) b = dep;
  const int bm = ok ? b : 0;  // arrivals moved
  float* const col = mix_slot(m, bin, 0, c);
  const float* top = col + (size_t)(dep - 1) * MIX_PL;  // arrival i in slot dep - 1 - i
  auto key = [&](int i) { return __float_as_int(top[MIX_KEY - (ptrdiff_t)i * MIX_PL]); };
  // the first ARR_KR keys in registers (all loads in flight together), the rest read as needed
  int kr[ARR_KR];
#pragma unroll
  for (int i = 0; i < ARR_KR; ++i) kr[i] = i < bm ? key(i) : 0x7fffffff;
  auto rank_of = [&](int ki) {
    int r = 0;
#pragma unroll
    for (int l = 0; l < ARR_KR; ++l) r += kr[l] < ki ? 1 : 0;
    for (int l = ARR_KR; l < bm; ++l) r += key(l) < ki ? 1 : 0;
    return r;
  };
  auto move = [&](int i, int dst_slot, float4 (&w)[2]) {
    const float4* src = reinterpret_cast<const float4*>(top - (size_t)i * MIX_PL);
    w[0] = src[0];
    w[1] = src[1];
    (void)dst_slot;
  };
#pragma unroll
  for (int h = 0; h < ARR_KR; h += ARR_BATCH) {
    int dl[ARR_BATCH];
    float4 w[ARR_BATCH][2];
#pragma unroll
    for (int u = 0; u < ARR_BATCH; ++u) {
      dl[u] = h + u < bm ? j + rank_of(kr[h + u]) : -1;
      if (dl[u] >= 0) move(h + u, dl[u], w[u]);
    }
#pragma unroll
    for (int u = 0; u < ARR_BATCH; ++u)
      if (dl[u] >= 0) {
        float4* dst = reinterpret_cast<float4*>(col + (size_t)dl[u] * MIX_PL);
        dst[0] = w[u][0];
        dst[1] = w[u][1];
      }
  }
  for (int i = ARR_KR; i < bm; ++i) {
    float4 w[2];
    const int dl = j + rank_of(key(i));
    move(i, dl, w);
    float4* dst = reinterpret_cast<float4*>(col + (size_t)dl * MIX_PL);
    dst[0] = w[0];
    dst[1] = w[1];
  }
  const int nn = ok ? j + b : j;
  m.cnt[bin * MIX_TC + c] = nn;
  m.acnt[bin * MIX_TC + c] = 0;
  // room for the next step: count + 2 x arrivals, maximum over the bin
  int need = nn + 2 * b;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) need = max(need, __shfl_xor_sync(0xffffffffu, need, o));
  if ((c & 31) == 0) wmax[c >> 5] = need;
  __syncthreads();
  if (c == 0) {
    for (int w = 1; w < MIX_TC / 32; ++w) need = max(need, wmax[w]);
    m.bneed[bin] = need;
    if (8 * (long long)need > 7 * (long long)dep) atomicOr(m.grow, 1);
  }
}

void mix_migrate2d(const Dev2D& d, cudaStream_t s) { k_mix_arrive<<<d.m.nbin, MIX_TC, 0, s>>>(d); }

// copy of every column (cnt[bin][c] slots, all planes) from another layout into d.m's
__global__ void __launch_bounds__(MIX_TC) k_mix_relayout(Dev2D d, const float* from_P, const long long* from_boff) {
  const Mix2D& m = d.m;
  const int bin = blockIdx.x, c = threadIdx.x;
  const int n = m.cnt[bin * MIX_TC + c];
  const float4* src = reinterpret_cast<const float4*>(from_P + ((size_t)from_boff[bin] * MIX_TC + c) * MIX_W);
  float4* dst = reinterpret_cast<float4*>(mix_slot(m, bin, 0, c));
  for (int k = 0; k < n; ++k) {
    const size_t o = (size_t)k * (MIX_PL / 4);
    const float4 a = src[o], b = src[o + 1];
    dst[o] = a;
    dst[o + 1] = b;
  }
}

void mix_relayout2d(const Dev2D& d, const float* from_P, const long long* from_boff, cudaStream_t s) {
  k_mix_relayout<<<d.m.nbin, MIX_TC, 0, s>>>(d, from_P, from_boff);
}

int mix_initial_depth(double n, double c_dt_dx) {
  // count with a 25 % rise and 6 standard deviations of Poisson noise, plus room for the arrivals
  // of the first steps (a particle crosses a face with probability <= c dt / dx per dimension)
  const double arr = 0.5 * n * (c_dt_dx < 1.0 ? c_dt_dx : 1.0) + 4.0 * std::sqrt(n);
  const double dep = 1.25 * n + 6.0 * std::sqrt(n) + 2.0 * arr + 16.0;
  int k = ((int)std::ceil(dep) + 7) & ~7;
  return k > MIX_MAX_DEPTH ? MIX_MAX_DEPTH : k;
}

// ---------------------------------------------------------------------------
// reference layout -> columns: thread c copies the particles of cell c, which are
// contiguous in the cell-sorted row (cumcnt gives the range)
// ---------------------------------------------------------------------------
// One CTA per tile.  For each of the tile's 16 bucket rows, the 16 cells' particles are one
// contiguous range of the AoS row; the CTA reads that range with consecutive threads on
// consecutive words (coalesced), finds each word's cell among the 16 (cumcnt), and stores the
// converted component into the cell's column.
__global__ void __launch_bounds__(MIX_TC) k_mix_put(Dev2D d, const double* aos, int ndim, int np_host, int isp,
                                                   int ty0) {
  __shared__ int scc[MIX_TS][MIX_TS + 1];
  const Mix2D& m = d.m;
  const Grid2D g = d.g;
  const int tx = blockIdx.x, ty = ty0 + blockIdx.y;
  const int bin = (ty * m.ntx + tx) * d.ph.nsp + isp;
  const int c = threadIdx.x;
  const int dep = m.bdep[bin];
  for (int t = c; t < MIX_TS * (MIX_TS + 1); t += MIX_TC) {
    const int ly = t / (MIX_TS + 1), q = t - ly * (MIX_TS + 1);
    scc[ly][q] = d.cc[((size_t)isp * g.ny + ty * MIX_TS + ly) * (g.nx + 1) + tx * MIX_TS + q];
  }
  __syncthreads();
  {
    const int lx = c & (MIX_TS - 1), ly = c >> 4;
    int n = scc[ly][lx + 1] - scc[ly][lx];
    if (n > dep) {
      atomicOr(d.err, EB_CAPACITY);
      n = dep;
    }
    m.cnt[bin * MIX_TC + c] = n;
  }
  const double dxi = d.ph.d_delx;
  float* const col0 = mix_slot(m, bin, 0, 0);
  for (int ly = 0; ly < MIX_TS; ++ly) {
    const int first = scc[ly][0];
    const long long nw = (long long)(scc[ly][MIX_TS] - first) * ndim;
    const double* rowp = aos + ((size_t)((ty - ty0) * MIX_TS + ly) * np_host + first) * ndim;
    const int gy = ty * MIX_TS + ly;
    if (ndim == 6) {
      // two words of a particle per thread ((x, y), (ux, uy) or (uz, id)): each warp reads 512
      // contiguous bytes of the row with 16-byte loads -- whole lines, for a host array read in
      // place over the host link -- and writes the matching part of the slot
      const int n2 = (scc[ly][MIX_TS] - first) * 3;
      // each warp's 512 bytes start on a 128-byte line of the host array: w2 = 0 lies `skew`
      // 16-byte units above a line start, so the loop starts that many units early
      const int skew = (int)(((size_t)rowp >> 4) & 7);
      for (int w2 = c - skew; w2 < n2; w2 += MIX_TC) {
        if (w2 < 0) continue;
        const int pl = w2 / 3, part = w2 - pl * 3;
        const int p = first + pl;
        int lx = 0;
#pragma unroll
        for (int step = 8; step > 0; step >>= 1)
          if (scc[ly][lx + step] <= p) lx += step;
        const int k = p - scc[ly][lx];
        if (k >= dep) continue;
        const double2 v = reinterpret_cast<const double2*>(rowp)[w2];
        float* o = col0 + (size_t)k * MIX_PL + (ly * MIX_TS + lx) * MIX_W;
        if (part == 0) {
          const int gx = tx * MIX_TS + lx;
          *reinterpret_cast<float2*>(o + MIX_OX) =
              make_float2(fminf((float)(v.x * dxi - (double)(g.nxgs + gx)), 0.99999994f),
                          fminf((float)(v.y * dxi - (double)(g.nygs + gy)), 0.99999994f));
        } else if (part == 1) {
          *reinterpret_cast<float2*>(o + MIX_UX) = make_float2((float)v.x, (float)v.y);
        } else {
          const long long id = __double_as_longlong(v.y);
          *reinterpret_cast<float4*>(o + MIX_UZ) =
              make_float4((float)v.x, __int_as_float((int)(unsigned)(id & 0xffffffffll)),
                          __int_as_float((int)(unsigned)((unsigned long long)id >> 32)), 0.f);
        }
      }
      continue;
    }
    for (long long w = c; w < nw; w += MIX_TC) {
      const int pl = (int)(w / ndim), comp = (int)(w - (long long)pl * ndim);
      const int p = first + pl;
      int lx = 0;
#pragma unroll
      for (int step = 8; step > 0; step >>= 1)
        if (scc[ly][lx + step] <= p) lx += step;
      const int k = p - scc[ly][lx];
      if (k >= dep || comp > 5) continue;
      const double a = rowp[w];
      float* o = col0 + (size_t)k * MIX_PL + (ly * MIX_TS + lx) * MIX_W;
      const int gx = tx * MIX_TS + lx;
      // offsets in [0, 1): a position within 2^-25 cells below a face rounds up to 1 in FP32
      if (comp == 0) o[MIX_OX] = fminf((float)(a * dxi - (double)(g.nxgs + gx)), 0.99999994f);
      else if (comp == 1) o[MIX_OY] = fminf((float)(a * dxi - (double)(g.nygs + gy)), 0.99999994f);
      else if (comp == 2) o[MIX_UX] = (float)a;
      else if (comp == 3) o[MIX_UY] = (float)a;
      else if (comp == 4) o[MIX_UZ] = (float)a;
      else {
        const long long id = __double_as_longlong(a);
        o[MIX_IDLO] = __int_as_float((int)(unsigned)(id & 0xffffffffll));
        o[MIX_IDHI] = __int_as_float((int)(unsigned)((unsigned long long)id >> 32));
      }
    }
    if (ndim <= 5) {  // no id words in the input: ids are zero
      const int n = scc[ly][MIX_TS] - first;
      for (int pl = c; pl < n; pl += MIX_TC) {
        const int p = first + pl;
        int lx = 0;
#pragma unroll
        for (int step = 8; step > 0; step >>= 1)
          if (scc[ly][lx + step] <= p) lx += step;
        const int k = p - scc[ly][lx];
        if (k >= dep) continue;
        float* o = col0 + (size_t)k * MIX_PL + (ly * MIX_TS + lx) * MIX_W;
        o[MIX_IDLO] = 0.f;
        o[MIX_IDHI] = 0.f;
      }
    }
  }
}

// per bin, the largest particle count of its cells in the reference-layout cumcnt (d.cc)
__global__ void __launch_bounds__(MIX_TC) k_mix_binmax(Dev2D d) {
  __shared__ int wmax[MIX_TC / 32];
  const Mix2D& m = d.m;
  const Grid2D g = d.g;
  const int bin = blockIdx.x;
  const int nsp = d.ph.nsp;
  const int tile = bin / nsp, isp = bin - tile * nsp;
  const int tx = tile % m.ntx, ty = tile / m.ntx;
  const int c = threadIdx.x;
  const int gx = tx * MIX_TS + (c & (MIX_TS - 1)), gy = ty * MIX_TS + (c >> 4);
  const int* ccr = d.cc + ((size_t)isp * g.ny + gy) * (g.nx + 1);
  int v = ccr[gx + 1] - ccr[gx];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((c & 31) == 0) wmax[c >> 5] = v;
  __syncthreads();
  if (c == 0) {
    for (int w = 1; w < MIX_TC / 32; ++w) v = max(v, wmax[w]);
    m.bneed[bin] = v;
  }
}

void mix_binmax2d(const Dev2D& d, cudaStream_t s) { k_mix_binmax<<<d.m.nbin, MIX_TC, 0, s>>>(d); }

void mix_put2d(const Dev2D& d, const double* aos, int ndim, int np_host, int isp, int ty0, int nty,
               cudaStream_t s) {
  dim3 grid(d.m.ntx, nty);
  k_mix_put<<<grid, MIX_TC, 0, s>>>(d, aos, ndim, np_host, isp, ty0);
}

// ---------------------------------------------------------------------------
// columns -> reference layout: per-row exclusive scan of the column counts into
// cumcnt and np2, then each column is written at its cell's offset, column order
// kept inside the cell
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(32) k_mix_rowscan(Dev2D d) {
  const Mix2D& m = d.m;
  const int row = blockIdx.x;
  const int isp = row / d.g.ny, gy = row - isp * d.g.ny;
  const int lane = threadIdx.x;
  const int nx = d.g.nx;
  int* ccr = d.cc + (size_t)row * (nx + 1);
  const int ty = gy / MIX_TS, ly = gy % MIX_TS;
  int carry = 0;
  for (int k0 = 0; k0 < nx; k0 += 32) {
    const int gx = k0 + lane;
    int v = 0;
    if (gx < nx) {
      const int bin = (ty * m.ntx + gx / MIX_TS) * d.ph.nsp + isp;
      v = m.cnt[bin * MIX_TC + ly * MIX_TS + gx % MIX_TS];
    }
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (gx < nx) ccr[gx] = incl - v + carry;
    carry += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (lane == 0) {
    ccr[nx] = carry;
    d.np2[row] = carry;
  }
}

void mix_count_rows2d(const Dev2D& d, cudaStream_t s) { k_mix_rowscan<<<d.nrowjob, 32, 0, s>>>(d); }

// One CTA per tile, the reverse of k_mix_put: the tile's particles of each bucket row are
// written as one contiguous AoS range (cumcnt from k_mix_rowscan), consecutive threads on
// consecutive words.
__global__ void __launch_bounds__(MIX_TC) k_mix_get(Dev2D d, double* aos, int ndim, int np_host, int isp, int ty0) {
  __shared__ int scc[MIX_TS][MIX_TS + 1];
  const Mix2D& m = d.m;
  const Grid2D g = d.g;
  const int tx = blockIdx.x, ty = ty0 + blockIdx.y;
  const int bin = (ty * m.ntx + tx) * d.ph.nsp + isp;
  const int c = threadIdx.x;
  for (int t = c; t < MIX_TS * (MIX_TS + 1); t += MIX_TC) {
    const int ly = t / (MIX_TS + 1), q = t - ly * (MIX_TS + 1);
    scc[ly][q] = d.cc[((size_t)isp * g.ny + ty * MIX_TS + ly) * (g.nx + 1) + tx * MIX_TS + q];
  }
  __syncthreads();
  const double dx = d.ph.delx;
  const float* const col0 = mix_slot(m, bin, 0, 0);
  for (int ly = 0; ly < MIX_TS; ++ly) {
    const int first = scc[ly][0];
    int last = scc[ly][MIX_TS];
    if (last > np_host) {
      if (c == 0) atomicOr(d.err, EB_CAPACITY);
      last = np_host;
    }
    const long long nw = (long long)(last - first) * ndim;
    double* rowp = aos + ((size_t)((ty - ty0) * MIX_TS + ly) * np_host + (first > 0 ? first : 0)) * ndim;
    const int gy = ty * MIX_TS + ly;
    if (ndim == 6) {
      // two words of a particle per thread ((x, y), (ux, uy) or (uz, id)): each warp writes 512
      // contiguous bytes of the row with 16-byte stores -- whole lines, for a host array written
      // in place over the host link
      const int n2 = (last - first) * 3;
      const int skew = (int)(((size_t)rowp >> 4) & 7);  // whole 128-byte lines per warp, as in k_mix_put
      for (int w2 = c - skew; w2 < n2; w2 += MIX_TC) {
        if (w2 < 0) continue;
        const int pl = w2 / 3, part = w2 - pl * 3;
        const int p = first + pl;
        int lx = 0;
#pragma unroll
        for (int step = 8; step > 0; step >>= 1)
          if (scc[ly][lx + step] <= p) lx += step;
        const int k = p - scc[ly][lx];
        const float* o = col0 + (size_t)k * MIX_PL + (ly * MIX_TS + lx) * MIX_W;
        double2 v;
        if (part == 0) {
          const float2 f = *reinterpret_cast<const float2*>(o + MIX_OX);
          v = make_double2(((double)(g.nxgs + tx * MIX_TS + lx) + (double)f.x) * dx, ((double)(g.nygs + gy) + (double)f.y) * dx);
        } else if (part == 1) {
          const float2 f = *reinterpret_cast<const float2*>(o + MIX_UX);
          v = make_double2((double)f.x, (double)f.y);
        } else {
          const float4 f = *reinterpret_cast<const float4*>(o + MIX_UZ);
          const unsigned long long id = ((unsigned long long)(unsigned)__float_as_int(f.z) << 32) |
                                        (unsigned)__float_as_int(f.y);
          v = make_double2((double)f.x, __longlong_as_double((long long)id));
        }
        reinterpret_cast<double2*>(rowp)[w2] = v;
      }
      continue;
    }
    for (long long w = c; w < nw; w += MIX_TC) {
      const int pl = (int)(w / ndim), comp = (int)(w - (long long)pl * ndim);
      const int p = first + pl;
      int lx = 0;
#pragma unroll
      for (int step = 8; step > 0; step >>= 1)
        if (scc[ly][lx + step] <= p) lx += step;
      const int k = p - scc[ly][lx];
      const float* o = col0 + (size_t)k * MIX_PL + (ly * MIX_TS + lx) * MIX_W;
      const int gx = tx * MIX_TS + lx;
      double v;
      if (comp == 0) v = ((double)(g.nxgs + gx) + (double)o[MIX_OX]) * dx;
      else if (comp == 1) v = ((double)(g.nygs + gy) + (double)o[MIX_OY]) * dx;
      else if (comp == 2) v = (double)o[MIX_UX];
      else if (comp == 3) v = (double)o[MIX_UY];
      else if (comp == 4) v = (double)o[MIX_UZ];
      else if (comp == 5) {
        const unsigned long long id = ((unsigned long long)(unsigned)__float_as_int(o[MIX_IDHI]) << 32) |
                                      (unsigned)__float_as_int(o[MIX_IDLO]);
        v = __longlong_as_double((long long)id);
      } else {
        v = 0.0;
      }
      rowp[w] = v;
    }
  }
}

void mix_get2d(const Dev2D& d, double* aos, int ndim, int np_host, int isp, int ty0, int nty, cudaStream_t s) {
  dim3 grid(d.m.ntx, nty);
  k_mix_get<<<grid, MIX_TC, 0, s>>>(d, aos, ndim, np_host, isp, ty0);
}

// ---------------------------------------------------------------------------
// device loader: the same plasma as load_weibel2d_ppc (same Philox counters: row-local
// particle index k = cx*ppc + kk, row jj); copy kk of cell c goes to slot (kk, c)
// ---------------------------------------------------------------------------
__global__ void k_mix_load(Dev2D d, int ppc, unsigned long long seed, double drift, int axis, double u_thi,
                           double u_the) {
  const Mix2D& m = d.m;
  const Grid2D g = d.g;
  const int bin = blockIdx.x;
  const int nsp = d.ph.nsp;
  const int tile = bin / nsp, isp = bin - tile * nsp;
  const int tx = tile % m.ntx, ty = tile / m.ntx;
  const int s = blockIdx.y * blockDim.x + threadIdx.x;  // = kk * 256 + c
  const int c = s % MIX_TC, kk = s / MIX_TC;
  const int dep = m.bdep[bin];
  if (kk == 0) m.cnt[bin * MIX_TC + c] = ppc < dep ? ppc : dep;
  if (kk >= ppc || kk >= dep) return;
  const int lx = c & (MIX_TS - 1), ly = c >> 4;
  const int cx = tx * MIX_TS + lx, jj = ty * MIX_TS + ly;
  const int k = cx * ppc + kk;
  const uint2 key = make_uint2((unsigned)seed, (unsigned)(seed >> 32));
  const uint4 rp = philox4x32(make_uint4((unsigned)k, (unsigned)jj, 0u, 0u), key);
  const uint4 r1 = philox4x32(make_uint4((unsigned)k, (unsigned)jj, 1u + 2u * isp, 0u), key);
  const uint4 r2 = philox4x32(make_uint4((unsigned)k, (unsigned)jj, 2u + 2u * isp, 0u), key);
  float* const o = mix_slot(m, bin, kk, c);
  float ox = (float)(1.0 - u01(rp.x, rp.y)), oy = (float)(1.0 - u01(rp.z, rp.w));
  if (ox >= 1.f) ox = 0.f;
  if (oy >= 1.f) oy = 0.f;
  o[MIX_OX] = ox;
  o[MIX_OY] = oy;
  const double sd = isp == 0 ? u_thi : u_the;
  const double twopi = 6.283185307179586;
  const double a1 = u01(r1.x, r1.y), b1 = u01(r1.z, r1.w), a2 = u01(r2.x, r2.y), b2 = u01(r2.z, r2.w);
  const double rad1 = sqrt(-2.0 * log(a1)), rad2 = sqrt(-2.0 * log(a2));
  double u[3] = {sd * rad1 * cos(twopi * b1), sd * rad1 * sin(twopi * b1), sd * rad2 * cos(twopi * b2)};
  if (isp == 1 && drift != 0.0) u[axis] += (k % 2 == 0) ? drift : -drift;
  o[MIX_UX] = (float)u[0];
  o[MIX_UY] = (float)u[1];
  o[MIX_UZ] = (float)u[2];
  const long long id = -((long long)jj * g.nx * ppc + k + 1);
  o[MIX_IDLO] = __int_as_float((int)(unsigned)(id & 0xffffffffll));
  o[MIX_IDHI] = __int_as_float((int)(unsigned)((unsigned long long)id >> 32));
}

void mix_load_weibel2d(const Dev2D& d, int ppc, unsigned long long seed, double drift, int drift_axis,
                       double u_thi, double u_the, cudaStream_t s) {
  dim3 grid(d.m.nbin, (MIX_TC * ppc + 255) / 256);  // bins on x (the y extent is limited to 65535)
  k_mix_load<<<grid, 256, 0, s>>>(d, ppc, seed, drift, drift_axis, u_thi, u_the);
}

// kinetic energy sums in FP64 over the FP32 momenta (2d/proj/weibel/app.f90:507-519)
__global__ void __launch_bounds__(MIX_TC) k_mix_energy(Dev2D d) {
  __shared__ double sh[MIX_TC];
  const Mix2D& m = d.m;
  const int isp = blockIdx.y;
  const double c = d.ph.c, rr = d.ph.r[isp];
  double v = 0.0;
  for (int tile = blockIdx.x; tile < m.ntile; tile += gridDim.x) {
    const int bin = tile * d.ph.nsp + isp;
    const int n = m.cnt[bin * MIX_TC + threadIdx.x];
    const float* col = mix_slot(m, bin, 0, threadIdx.x);
    for (int k = 0; k < n; ++k) {
      const float* o = col + (size_t)k * MIX_PL;
      const double a = o[MIX_UX], b = o[MIX_UY], e = o[MIX_UZ];
      v += rr * (sqrt(1.0 + (a * a + b * b + e * e) / (c * c)) - 1.0);
    }
  }
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int w = MIX_TC / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) d.partials[((size_t)isp * d.nred + blockIdx.x) * 2] = sh[0];
}

void mix_energy2d(const Dev2D& d, cudaStream_t s) {
  cudaMemsetAsync(d.partials, 0, sizeof(double) * 2 * 3 * (size_t)d.nred, s);
  const int nb = d.nred < d.m.ntile ? d.nred : d.m.ntile;
  k_mix_energy<<<dim3(nb, d.ph.nsp), MIX_TC, 0, s>>>(d);
  fast::energy_fields_fin2d(d, s);
}

// ---------------------------------------------------------------------------
// mom_calc__accl + mom_calc__nvt (2d/common/mom_calc.f90:48-249) on the column layout:
// one CTA per (tile, species), thread c walks the column of cell c.  The half-step Boris
// push of mom_calc__accl (time step halved by mom_calc__init, :36) runs in FP32 on the
// cell-centred fields; the seven moments of the particle go into the thread's registers
// over the 3 x 3 nodes its cell can reach (node ih = floor(x/dx - 0.5) is cell i - 1 or i),
// then into the tile's 18 x 18 node patch (FP32 shared atomics) and once per node into the
// FP64 global moments.  The state is not modified (the reference writes gp, which the next
// step overwrites).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(MIX_TC) k_mix_mom(Dev2D d, double* mom) {
  __shared__ __align__(16) float4 sfa[TT * TT];  // (Bx, By, Bz, Ex) at cell centres, local cells -1..16
  __shared__ __align__(8) float2 sfb[TT * TT];   // (Ey, Ez)
  __shared__ float macc[7][TT][TT];              // node patch: local node xl = node index - 16 tx
  const Mix2D& m = d.m;
  const Grid2D g = d.g;
  const int tile = blockIdx.x, isp = blockIdx.y;
  const int tx = tile % m.ntx, ty = tile / m.ntx;
  const int c = threadIdx.x;
  for (int k = c; k < TT * TT; k += MIX_TC) {
    const int r = k / TT, cc = k % TT;  // local cell (cc - 1, r - 1), field index + 2
    const int fi = tx * MIX_TS + cc + 1, fj = ty * MIX_TS + r + 1;
    const double* U = d.uf + (size_t)fj * g.fp + fi;
#define UF(comp, di, dj) U[(size_t)(comp) * g.fplane + (size_t)(dj) * g.fp + (di)]
    sfa[k] = make_float4((float)(0.5 * (UF(0, 0, 0) + UF(0, 0, 1))), (float)(0.5 * (UF(1, 0, 0) + UF(1, 1, 0))),
                         (float)(0.25 * (UF(2, 0, 0) + UF(2, 1, 0) + UF(2, 0, 1) + UF(2, 1, 1))),
                         (float)(0.5 * (UF(3, 0, 0) + UF(3, 1, 0))));
    sfb[k] = make_float2((float)(0.5 * (UF(4, 0, 0) + UF(4, 0, 1))), (float)UF(5, 0, 0));
#undef UF
  }
  for (int k = c; k < 7 * TT * TT; k += MIX_TC) (&macc[0][0][0])[k] = 0.f;
  __syncthreads();

  const int bin = tile * d.ph.nsp + isp;
  const int n = m.cnt[bin * MIX_TC + c];
  const float* col = mix_slot(m, bin, 0, c);
  const double hdt = d.ph.delt * 0.5;
  const float fac1 = (float)(d.ph.q[isp] / d.ph.r[isp] * 0.5 * hdt);
  const float fac2 = (float)(d.ph.q[isp] * hdt / d.ph.r[isp]);
  const float txxx = fac1 * fac1;
  const float cl = m.k_c, ic2 = m.k_ic2;
  const int lx = c & (MIX_TS - 1), ly = c >> 4;
  const int f0 = ly * TT + lx;
  float acc[7][3][3];
#pragma unroll
  for (int l = 0; l < 7; ++l)
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int a = 0; a < 3; ++a) acc[l][b][a] = 0.f;
  for (int k = 0; k < n; ++k) {
    const float* o = col + (size_t)k * MIX_PL;
    const float ox = o[MIX_OX], oy = o[MIX_OY];
    const float ux0 = o[MIX_UX], uy0 = o[MIX_UY], uz0 = o[MIX_UZ];
    const float sx0 = 0.5f * (1.f - ox) * (1.f - ox), sx1 = 0.75f - (ox - 0.5f) * (ox - 0.5f), sx2 = 0.5f * ox * ox;
    const float sy0 = 0.5f * (1.f - oy) * (1.f - oy), sy1 = 0.75f - (oy - 0.5f) * (oy - 0.5f), sy2 = 0.5f * oy * oy;
    float f[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int jy = 0; jy < 3; ++jy) {
      const float wy = jy == 0 ? sy0 : (jy == 1 ? sy1 : sy2);
#pragma unroll
      for (int jx = 0; jx < 3; ++jx) {
        const float w = wy * (jx == 0 ? sx0 : (jx == 1 ? sx1 : sx2));
        const float4 a = sfa[f0 + jy * TT + jx];
        const float2 b = sfb[f0 + jy * TT + jx];
        f[0] = fmaf(w, a.x, f[0]);
        f[1] = fmaf(w, a.y, f[1]);
        f[2] = fmaf(w, a.z, f[2]);
        f[3] = fmaf(w, a.w, f[3]);
        f[4] = fmaf(w, b.x, f[4]);
        f[5] = fmaf(w, b.y, f[5]);
      }
    }
    const float bpx = f[0], bpy = f[1], bpz = f[2], epx = f[3], epy = f[4], epz = f[5];
    float u1 = ux0 + fac1 * epx, u2 = uy0 + fac1 * epy, u3 = uz0 + fac1 * epz;
    const float g2 = cl * cl + u1 * u1 + u2 * u2 + u3 * u3;
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
    const float ux = u1 + fac1 * epx, uy = u2 + fac1 * epy, uz = u3 + fac1 * epz;
    const float gam = rsqrtf(1.f + (ux * ux + uy * uy + uz * uz) * ic2);
    // linear weights over nodes i-1, i, i+1 (and j-1, j, j+1)
    const float hx = ox - 0.5f, hy = oy - 0.5f;
    const float wx[3] = {hx < 0.f ? -hx : 0.f, hx < 0.f ? hx + 1.f : 1.f - hx, hx < 0.f ? 0.f : hx};
    const float wy[3] = {hy < 0.f ? -hy : 0.f, hy < 0.f ? hy + 1.f : 1.f - hy, hy < 0.f ? 0.f : hy};
    const float pre[7] = {1.f, ux * gam, uy * gam, uz * gam, ux * ux * gam, uy * uy * gam, uz * uz * gam};
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const float w = wx[a] * wy[b];
#pragma unroll
        for (int l = 0; l < 7; ++l) acc[l][b][a] = fmaf(pre[l], w, acc[l][b][a]);
      }
  }
  if (n > 0) {
#pragma unroll
    for (int l = 0; l < 7; ++l)
#pragma unroll
      for (int b = 0; b < 3; ++b)
#pragma unroll
        for (int a = 0; a < 3; ++a) atomicAdd(&macc[l][ly + b][lx + a], acc[l][b][a]);
  }
  __syncthreads();
  const int nxm = g.nx + 2, nym = g.ny + 2;
  for (int k = c; k < TT * TT; k += MIX_TC) {
    const int yl = k / TT, xl = k % TT;
    const size_t in = (size_t)tx * MIX_TS + xl, jn = (size_t)ty * MIX_TS + yl;
    double* out = mom + 7 * (in + (size_t)nxm * (jn + (size_t)nym * isp));
#pragma unroll
    for (int l = 0; l < 7; ++l) {
      const float v = macc[l][yl][xl];
      if (v != 0.f) atomicAdd(out + l, (double)v);
    }
  }
}

void mix_moments2d(const Dev2D& d, double* mom, cudaStream_t s) {
  cudaMemsetAsync(mom, 0, sizeof(double) * 7 * (size_t)(d.g.nx + 2) * (d.g.ny + 2) * d.ph.nsp, s);
  k_mix_mom<<<dim3(d.m.ntile, d.ph.nsp), MIX_TC, 0, s>>>(d, mom);
  bc_mom2d(d, mom, s);
}

int mix_setup2d(const Dev2D& d, void* out) {
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
  if (r != CUDA_SUCCESS) return -2;
  if (cudaFuncSetAttribute(k_mix_push2<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, PUSH2_SMEM) !=
          cudaSuccess ||
      cudaFuncSetAttribute(k_mix_push2<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, PUSH2_SMEM) !=
          cudaSuccess ||
      cudaFuncSetAttribute(k_mix_push2<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, PUSH2_SMEM) !=
          cudaSuccess ||
      cudaFuncSetAttribute(k_mix_push2<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, PUSH2_SMEM) !=
          cudaSuccess)
    return -3;

  return 0;
}

}  // namespace wpic
