// Mixed-precision 3D path: particles stored as integer cell (implicit in their column) plus
// three FP32 offsets; FP32 push, gather and Esirkepov deposition; FP32 currents summed exactly
// in fixed point and converted to FP64 global J; FP64 field state and solver (the FP64 3D
// kernels of fp3d.cuh).
//
// Storage: per (8 x 8 x 4-cell tile, species) bin, one column of slots per cell (Mix3D in
// wpic_internal.h).  One CTA of 256 threads per tile runs particle__solv and ele_cur fused
// (3d/common/particle.f90:52-233, 3d/common/field.f90:211-406), thread c walking the column of
// cell c:
//  * the tile's E/B (12 x 11 x 7 nodes x 6 components, FP64) arrives in shared memory by one
//    TMA tensor load and is averaged to the cell centres of cells -1 .. T in FP32;
//  * each particle is pushed, moved in split form (cell + offset) and written back in place
//    (the column compacted) or, when it changes cell, to the top of its new cell's column;
//  * the Esirkepov current of a particle that stays in its cell goes into the thread's
//    registers: the support is the cell's 3 x 3 x 3 nodes, 2 x 3 x 3 values per component,
//    flushed every 32 iterations into the tile's fixed-point current (exact integer atomics);
//  * a particle that changes cell has a 4-node support along the axes it crosses; it is queued
//    per warp and deposited 32 at a time, one lane per particle, straight into the tile's
//    fixed-point current;
//  * the tile current is added once into the global fixed-point current.
// The periodic wraps of boundary_periodic__particle_x/_yz are integer cell arithmetic; the
// conducting walls of 3d/proj/reconnection and the shock window's wall and injection end act
// between the move and the deposit, as those drivers order their x boundary before the field
// solve.  A second kernel moves the arrivals to just above each column's stayers in a fixed
// key order (direction of arrival, then slot in the source column), so a step is bitwise
// reproducible -- the reference's scheme of arrivals filling a row's free slots
// (3d/common/boundary_periodic.f90:104-455) applied to a cell column.
#include <cuda.h>

#include <cmath>

#include "common.cuh"
#include "mixed_common.cuh"

namespace wpic {

namespace {

constexpr int TX = M3_TX, TY = M3_TY, TZ = M3_TZ, TC = M3_TC;
constexpr int FX = TX + 2, FY = TY + 2, FZ = TZ + 2;  // centred fields of local cells -1 .. T
constexpr int FN = FX * FY * FZ;
// TMA box of FP64 nodes: field columns cx0 .. cx0+11 (an even start, as the tensor copy's
// 16-byte rule asks), rows cy0+1 .. cy0+11, layers cz0+1 .. cz0+7, six components
constexpr int SX = 12, SY = 11, SZ = 7;
constexpr int STAGE_BYTES = 6 * SZ * SY * SX * 8;
// current patch: nodes at local offsets -2 .. T+1, two int32 planes (hi, lo) per component
constexpr int JX = TX + 4, JY = TY + 4, JZ = TZ + 4;
constexpr int JN = JX * JY * JZ;
constexpr int PATCH_BYTES = 2 * 3 * JN * 4;
constexpr int PF = 4;  // particles in flight per thread (shared-memory ring)
constexpr int RING_BYTES = PF * M3_W * TC * 4;
constexpr int LQ = 64;                       // leaver queue entries per warp
constexpr int LQW = 7;                       // 32-bit words per entry
constexpr int LQ_BYTES = (TC / 32) * LQW * LQ * 4;
constexpr int FLUSH_EVERY = 32;  // iterations between flushes of the register current
constexpr unsigned long long kSpinLimit = 1ull << 22;

static_assert(PATCH_BYTES + LQ_BYTES <= STAGE_BYTES, "the leaver queue lives behind the patch");

// dynamic shared memory: TMA staging (later the current patch + leaver queues), centred
// fields, particle ring, pending leavers
constexpr int OFF_STAGE = 0;
constexpr int OFF_SFA = (STAGE_BYTES + 127) / 128 * 128;
constexpr int OFF_SFB = OFF_SFA + FN * 16;
constexpr int OFF_RING = OFF_SFB + FN * 8;
constexpr int OFF_PEND = OFF_RING + RING_BYTES;

// a leaver of the push waiting for its slot (one per thread): the slot's 8 words, its arrival key
// and its new column (3 x 3 x 3 neighbourhood tile, species, cell)
struct Pending3 {
  float4 w[TC][2];
  int key[TC];
  int dst[TC];
};
constexpr int PUSH_SMEM = OFF_PEND + (int)sizeof(Pending3);

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

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
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar) {
  for (unsigned long long it = 0; it < kSpinLimit; ++it)
    if (mbar_try_wait(bar, 0)) return true;
  return false;
}
// TMA: 4D box (x = field column, y = row, z = layer, w = component) into shared memory
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* tm, int x, int y, int z, int w,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(smem_u32(dst)),
      "l"(tm), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ void ffma2_into(float& a0, float& a1, float x0, float x1, float y0, float y1) {
  const float2 r = __ffma2_rn(make_float2(x0, x1), make_float2(y0, y1), make_float2(a0, a1));
  a0 = r.x;
  a1 = r.y;
}

// p = old offset + displacement (cell units, |displacement| < 1): new cell increment and offset in
// [0, 1).  A step a hair below the lower face, where p + 1 rounds to 1, keeps the particle at
// offset 0 of its old cell.
__device__ __forceinline__ void split_move(float p, float& on, int& inc, int* err) {
  if (p >= 1.f) { on = p - 1.f; inc = 1; }
  else if (p < 0.f) { on = p + 1.f; inc = -1; }
  else { on = p; inc = 0; }
  if (on >= 1.f) { on = 0.f; inc += 1; }
  if (!(on >= 0.f && on < 1.f)) {
    atomicOr(err, EB_MOVED_TOO_FAR);  // moved a full cell or more (c dt >= dx), or not finite
    on = fminf(fmaxf(on, 0.f), 0.99999994f);
    if (!(on >= 0.f)) on = 0.f;
  }
}

// Mirror image X' = 2 W - X of the position X = cell + off about W = wc + wf (wf in [0, 1)),
// in split form: the integer parts cancel exactly and only the fractions are rounded.
__device__ __forceinline__ void reflect_split(int& cell, float& off, int wc, float wf) {
  const float r = (wf - off) + wf;  // in (-1, 2)
  const float fr = floorf(r);
  cell = 2 * wc - cell + (int)fr;
  off = r - fr;
  if (off >= 1.f) { off = 0.f; cell += 1; }
}

// Esirkepov current of one particle (3d/common/field.f90:331-381, the factored form) added to
// the tile patch in fixed point.  o = old offsets, p = new offsets in the new cell, inc = cell
// change per axis, (lx, ly, lz) = the old cell in the tile.  Along every axis the support of s0
// and s1 is 3 nodes, 4 when the particle changes cell, starting at node offset lo - 2.
__device__ __forceinline__ void deposit_general(const float o[3], const float p[3], const int inc[3], int lx, int ly,
                                                int lz, float qdd, int* jhi, int* jlo, float s1, float is1,
                                                float s2) {
  const float third = 1.0f / 3.0f;
  float s0w[3][4], dsw[3][4], pre[3][3];
  int lo[3], wd[3];
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    const float om = o[m];
    const float s0[5] = {0.f, 0.5f * (1.f - om) * (1.f - om), 0.75f - (om - 0.5f) * (om - 0.5f), 0.5f * om * om, 0.f};
    float ds[5];
    shape_diff5(om, p[m], inc[m], ds);
    lo[m] = inc[m] < 0 ? 0 : 1;
    wd[m] = inc[m] != 0 ? 4 : 3;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      s0w[m][i] = lo[m] == 0 ? s0[i] : s0[i + 1];
      dsw[m][i] = lo[m] == 0 ? ds[i] : ds[i + 1];
    }
    pre[m][0] = -dsw[m][0];
    pre[m][1] = pre[m][0] - dsw[m][1];
    pre[m][2] = pre[m][1] - dsw[m][2];
  }
#pragma unroll
  for (int comp = 0; comp < 3; ++comp) {
    const int t1 = comp == 0 ? 1 : 0;  // transverse axes t1 (jw) and t2 (kw)
    const int t2 = comp == 2 ? 1 : 2;
    const int ea = (comp == 0 ? lx : comp == 1 ? ly : lz) + lo[comp] + 1;  // own axis: edge aw at ea + aw
    const int e1 = (t1 == 0 ? lx : ly) + lo[t1];
    const int e2 = (t2 == 1 ? ly : lz) + lo[t2];
    // kw runs as a loop (the unrolled 4 x 4 x 3 sites per component made this function the
    // largest part of the kernel's code, and the particle loop around it missed the
    // instruction cache); s0w[t2][kw] and dsw[t2][kw] are selected, not indexed
#pragma unroll 1
    for (int kw = 0; kw < wd[t2]; ++kw) {
      const float s0k = kw == 0 ? s0w[t2][0] : kw == 1 ? s0w[t2][1] : kw == 2 ? s0w[t2][2] : s0w[t2][3];
      const float dsk = kw == 0 ? dsw[t2][0] : kw == 1 ? dsw[t2][1] : kw == 2 ? dsw[t2][2] : dsw[t2][3];
#pragma unroll
      for (int jw = 0; jw < 4; ++jw) {
        if (jw >= wd[t1]) continue;
        const float dstmp = ((s0w[t1][jw] + 0.5f * dsw[t1][jw]) * s0k +
                             (0.5f * s0w[t1][jw] + third * dsw[t1][jw]) * dsk) * qdd;
#pragma unroll
        for (int aw = 0; aw < 3; ++aw) {
          if (aw >= wd[comp] - 1) continue;
          int xl, yl, zl;
          if (comp == 0) { xl = ea + aw; yl = e1 + jw; zl = e2 + kw; }
          else if (comp == 1) { xl = e1 + jw; yl = ea + aw; zl = e2 + kw; }
          else { xl = e1 + jw; yl = e2 + kw; zl = ea + aw; }
          const int w = comp * JN + (zl * JY + yl) * JX + xl;
          fx_add(jhi + w, jlo + w, pre[comp][aw] * dstmp, s1, is1, s2);
        }
      }
    }
  }
}

// The register current of a thread's cell: for component x, jx[j][k] holds the pair of x edges
// (at local node offsets 0 and 1) for y node j - 1 and z node k - 1; likewise y (x node, z node)
// and z (x node, y node).
struct Cell3Current {
  float2 jx[3][3], jy[3][3], jz[3][3];
};

__device__ __forceinline__ void cell3_zero(Cell3Current& a) {
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int k = 0; k < 3; ++k) a.jx[j][k] = a.jy[j][k] = a.jz[j][k] = make_float2(0.f, 0.f);
}

__device__ __forceinline__ void cell3_flush(Cell3Current& a, int* jhi, int* jlo, int lx, int ly, int lz, float s1,
                                            float is1, float s2) {
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        // x edge at patch (lx + 2 + e, ly + 1 + j, lz + 1 + k); y edge at (lx + 1 + j, ly + 2 + e, lz + 1 + k);
        // z edge at (lx + 1 + j, ly + 1 + k, lz + 2 + e)
        const int wx = 0 * JN + ((lz + 1 + k) * JY + (ly + 1 + j)) * JX + (lx + 2 + e);
        const int wy = 1 * JN + ((lz + 1 + k) * JY + (ly + 2 + e)) * JX + (lx + 1 + j);
        const int wz = 2 * JN + ((lz + 2 + e) * JY + (ly + 1 + k)) * JX + (lx + 1 + j);
        fx_add(jhi + wx, jlo + wx, e ? a.jx[j][k].y : a.jx[j][k].x, s1, is1, s2);
        fx_add(jhi + wy, jlo + wy, e ? a.jy[j][k].y : a.jy[j][k].x, s1, is1, s2);
        fx_add(jhi + wz, jlo + wz, e ? a.jz[j][k].y : a.jz[j][k].x, s1, is1, s2);
      }
  cell3_zero(a);
}

// direction code d = (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1) of a move (13 = same cell) -> group 0..25
__device__ __forceinline__ int dir_group3(int d) { return d < 13 ? d : d - 1; }

// __cvta helpers come before the kernel; write_pending3 is defined inside the kernel as a lambda

}  // namespace

// ---------------------------------------------------------------------------
// fused push + deposit + column compaction, one CTA per tile, one thread per cell column
// VAY: the push of particle__solv_vay (3d/common/particle.f90:236-419)
// ---------------------------------------------------------------------------
template <bool VAY>
__global__ void __launch_bounds__(TC, 2) k_mix3_push(Dev3D d, Mix3Const k, const __grid_constant__ CUtensorMap tm) {
  extern __shared__ __align__(128) unsigned char smem[];
  double* const stage = reinterpret_cast<double*>(smem + OFF_STAGE);
  int* const jhi = reinterpret_cast<int*>(smem + OFF_STAGE);
  int* const jlo = jhi + 3 * JN;
  float* const lq = reinterpret_cast<float*>(smem + OFF_STAGE + PATCH_BYTES);  // [warp][word][LQ]
  float4* const sfa = reinterpret_cast<float4*>(smem + OFF_SFA);  // (Bx, By, Bz, Ex) at cell centres
  float2* const sfb = reinterpret_cast<float2*>(smem + OFF_SFB);  // (Ey, Ez)
  float* const ring = reinterpret_cast<float*>(smem + OFF_RING);  // [PF][8][TC]
  Pending3* const pend = reinterpret_cast<Pending3*>(smem + OFF_PEND);
  __shared__ __align__(8) unsigned long long bar;
  __shared__ int nb_bin[2][27], nb_dep[2][27];
  __shared__ long long nb_off[2][27];
  const Mix3D& m = d.m;
  const Grid3D g = d.g;
  const int tile = blockIdx.x;
  const int tx = tile % m.ntx, ty = (tile / m.ntx) % m.nty, tz = tile / (m.ntx * m.nty);
  const int cx0 = tx * TX, cy0 = ty * TY, cz0 = tz * TZ;
  const int c = threadIdx.x;
  const int lane = c & 31, warp = c >> 5;
  const int nsp = d.ph.nsp;
  const int bin0 = tile * nsp;
  const int n0 = m.cnt[bin0 * TC + c];
  const int ntot = n0 + (nsp > 1 ? m.cnt[(bin0 + 1) * TC + c] : 0);
  if (c < 2 * 27) {
    const int s = c / 27, q = c % 27;
    int ntx_ = tx + q % 3 - 1, nty_ = ty + (q / 3) % 3 - 1, ntz_ = tz + q / 9 - 1;
    if (ntx_ < 0) ntx_ += m.ntx; else if (ntx_ >= m.ntx) ntx_ -= m.ntx;
    if (nty_ < 0) nty_ += m.nty; else if (nty_ >= m.nty) nty_ -= m.nty;
    if (ntz_ < 0) ntz_ += m.ntz; else if (ntz_ >= m.ntz) ntz_ -= m.ntz;
    const int b = ((ntz_ * m.nty + nty_) * m.ntx + ntx_) * nsp + (s < nsp ? s : 0);
    nb_bin[s][q] = b;
    nb_dep[s][q] = m.bdep[b];
    nb_off[s][q] = m.boff[b];
  }
  // slot of flattened item t (species 0 items first): col[t >= n0] + t layers
  float* const col0 = mix3_slot(m, bin0, 0, c);
  float* const col1 = mix3_slot(m, bin0 + (nsp > 1 ? 1 : 0), 0, c) - (size_t)n0 * M3_PL;
  auto issue = [&](int t) {
    if (t < ntot) {
      const float* src = (t < n0 ? col0 : col1) + (size_t)t * M3_PL;
      float* dst = ring + ((t & (PF - 1)) * TC + c) * M3_W;
      cp_async16(dst, src);
      cp_async16(dst + 4, src + 4);
    }
    cp_async_commit();
  };
#pragma unroll
  for (int t = 0; t < PF; ++t) issue(t);
  if (c == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (c == 0) {
    mbar_expect_tx(&bar, (unsigned)STAGE_BYTES);
    tma_load_4d(stage, &tm, cx0, cy0 + 1, cz0 + 1, 0, &bar);
  }
  // every thread waits (bounded) for the tile; the CTA gives up together if any wait ran out
  const bool staged = mbar_wait_bounded(&bar);
  if (!__syncthreads_and(staged)) {
    if (c == 0) atomicOr(d.err, EB_STAGING_TIMEOUT);
    if (!staged) mbar_wait_bounded(&bar);  // second bounded wait for the copy in flight
    cp_async_wait<0>();
    return;
  }
  // cell-centred fields of local cells (a-1, b-1, cc-1) (3d/common/particle.f90:75-92), FP64 sums
  // rounded to FP32; staged node (sx, sy, sz) is field index (cx0 + sx, cy0 + 1 + sy, cz0 + 1 + sz)
  for (int idx = c; idx < FN; idx += TC) {
    const int a = idx % FX, b = (idx / FX) % FY, cc = idx / (FX * FY);
    const int sx = a + 1, sy = b, sz = cc;
    auto S = [&](int comp, int z, int y, int x) { return stage[((comp * SZ + z) * SY + y) * SX + x]; };
    const double bx = 2.5e-1 * (S(0, sz, sy, sx) + S(0, sz, sy + 1, sx) + S(0, sz + 1, sy, sx) + S(0, sz + 1, sy + 1, sx));
    const double by = 2.5e-1 * (S(1, sz, sy, sx) + S(1, sz, sy, sx + 1) + S(1, sz + 1, sy, sx) + S(1, sz + 1, sy, sx + 1));
    const double bz = 2.5e-1 * (S(2, sz, sy, sx) + S(2, sz, sy, sx + 1) + S(2, sz, sy + 1, sx) + S(2, sz, sy + 1, sx + 1));
    const double ex = 5e-1 * (S(3, sz, sy, sx) + S(3, sz, sy, sx + 1));
    const double ey = 5e-1 * (S(4, sz, sy, sx) + S(4, sz, sy + 1, sx));
    const double ez = 5e-1 * (S(5, sz, sy, sx) + S(5, sz + 1, sy, sx));
    sfa[idx] = make_float4((float)bx, (float)by, (float)bz, (float)ex);
    sfb[idx] = make_float2((float)ey, (float)ez);
  }
  __syncthreads();
  for (int idx = c; idx < 2 * 3 * JN; idx += TC) jhi[idx] = 0;
  __syncthreads();
  const float fs1 = m.fx_s1, fs2 = m.fx_s2, fis1 = m.fx_is1f;
  const int lx = c & (TX - 1), ly = (c >> 3) & (TY - 1), lz = c >> 6;
  const int ci = cx0 + lx;
  const float dtdx = k.dtdx, cl = k.c, ic2 = k.ic2;
  const float third = 1.0f / 3.0f;
  const int bc = d.ph.bc;
  const int f0 = (lz * FY + ly) * FX + lx;  // this cell's 3 x 3 x 3 centred-field stencil starts here
  Cell3Current acc;
  cell3_zero(acc);
  float* const myq = lq + warp * LQW * LQ;
  int qhead = 0, qtail = 0;  // the warp's leaver queue (warp-uniform)
  // deposit `cnt` queued leavers, one per lane (warp-uniform call)
  auto drain = [&](int cnt) {
    if (lane < cnt) {
      const int e = (qhead + lane) & (LQ - 1);
      const float o[3] = {myq[0 * LQ + e], myq[1 * LQ + e], myq[2 * LQ + e]};
      const float p[3] = {myq[3 * LQ + e], myq[4 * LQ + e], myq[5 * LQ + e]};
      const int pk = __float_as_int(myq[6 * LQ + e]);
      const int inc[3] = {(pk & 3) - 1, ((pk >> 2) & 3) - 1, ((pk >> 4) & 3) - 1};
      const int cc = pk >> 8;
      const float qdd = (pk >> 6) & 1 ? k.qdd[1] : k.qdd[0];
      deposit_general(o, p, inc, cc & (TX - 1), (cc >> 3) & (TY - 1), cc >> 6, qdd, jhi, jlo, fs1, fis1, fs2);
    }
    qhead += cnt;
    __syncwarp();
  };
  // the pending leaver of this thread (its slot returned by the last iteration's atomic): arrival
  // number pos of a column goes to slot depth - 1 - pos, its key beside it in the key array
  auto write_pending3 = [&](int pos) {
    const int dst = pend->dst[c];
    const int q = dst & 31, s = (dst >> 5) & 1, dlc = dst >> 8;
    const int dep = nb_dep[s][q];
    if (pos >= dep) {
      atomicOr(d.err, EB_CAPACITY);
      return;
    }
    const size_t slot = ((size_t)nb_off[s][q] + dep - 1 - pos) * TC + dlc;
    float4* io = reinterpret_cast<float4*>(m.P + slot * M3_W);
    io[0] = pend->w[c][0];
    io[1] = pend->w[c][1];
    m.K[slot] = pend->key[c];
  };
  int j0 = 0, j1 = 0;  // stayers kept so far per species (compacted in place)
  int ppos = -1;       // arrival number of the pending leaver parked in shared memory, -1 if none
  int tw = ntot;       // iterations of this warp: the largest column of its lanes
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) tw = max(tw, __shfl_xor_sync(0xffffffffu, tw, o));
  for (int t = 0; t < tw; ++t) {
    cp_async_wait<PF - 1>();
    bool leaver = false;
    float lo_[3], ln_[3];
    int linc[3];
    bool lsp1 = false;
    if (t < ntot) {
      const bool sp1 = t >= n0;
      const int kk = sp1 ? t - n0 : t;
      const float4* pb = reinterpret_cast<const float4*>(ring + ((t & (PF - 1)) * TC + c) * M3_W);
      const float4 pa = pb[0], pz = pb[1];
      const float o[3] = {pa.x, pa.y, pa.z};
      float ux = pa.w, uy = pz.x, uz = pz.y;
      const float idlo = pz.z, idhi = pz.w;
      const float fac1 = sp1 ? k.fac1[1] : k.fac1[0];
      const float fac2 = sp1 ? k.fac2[1] : k.fac2[0];
      const float qdd = sp1 ? k.qdd[1] : k.qdd[0];
      float w[3][3];
#pragma unroll
      for (int mm = 0; mm < 3; ++mm) {
        w[mm][0] = 0.5f * (1.f - o[mm]) * (1.f - o[mm]);
        w[mm][1] = 0.75f - (o[mm] - 0.5f) * (o[mm] - 0.5f);
        w[mm][2] = 0.5f * o[mm] * o[mm];
      }
      // gather (3d/common/particle.f90:120-170): 27 centred nodes, six components
      float f[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int c3 = 0; c3 < 3; ++c3)
#pragma unroll
        for (int b3 = 0; b3 < 3; ++b3) {
          const float wzy = w[2][c3] * w[1][b3];
#pragma unroll
          for (int a3 = 0; a3 < 3; ++a3) {
            const float wt = wzy * w[0][a3];
            const int n = f0 + (c3 * FY + b3) * FX + a3;
            const float4 A = sfa[n];
            const float2 B = sfb[n];
            ffma2_into(f[0], f[1], wt, wt, A.x, A.y);
            ffma2_into(f[2], f[3], wt, wt, A.z, A.w);
            ffma2_into(f[4], f[5], wt, wt, B.x, B.y);
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
        // Buneman-Boris (3d/common/particle.f90:182-205)
        const float txxx = fac1 * fac1;
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
      const float dsp = dtdx * ig;
      float on[3];
      int inc[3];
      split_move(o[0] + ux * dsp, on[0], inc[0], d.err);
      split_move(o[1] + uy * dsp, on[1], inc[1], d.err);
      split_move(o[2] + uz * dsp, on[2], inc[2], d.err);
      if (bc != BC_PERIODIC) {
        // the x boundary before the deposit, in split form.  Reconnection: particle_x
        // (3d/proj/reconnection/app.f90:103-108), reflection about the walls at cells 1 and nx-2
        // (nxs+1 and nxe-1), all three momentum components reversed
        // (3d/proj/reconnection/boundary_reconnection.f90:69-101).  Shock: boundary_shock__injection
        // (3d/proj/shock/app.f90:112-113, boundary_shock.f90:424-469), reflection about cell wx0 + 1
        // with the momenta reversed, and beyond xend: x -> 2 xend - x, u_x -> 2 u0 - u_x, u_y and u_z
        // reversed.
        int gxn = ci + inc[0];
        float X = on[0];
        bool flip = false;
        if (bc == BC_RECONNECTION) {
          if (gxn < 1) { reflect_split(gxn, X, 1, 0.f); flip = true; }
          else if (gxn >= g.nx - 2) { reflect_split(gxn, X, g.nx - 2, 0.f); flip = true; }
          if (flip) { ux = -ux; uy = -uy; uz = -uz; }
        } else {
          if (gxn < g.wx0 + 1) {
            reflect_split(gxn, X, g.wx0 + 1, 0.f);
            ux = -ux; uy = -uy; uz = -uz;
            flip = true;
          } else if (gxn > k.xend_cell || (gxn == k.xend_cell && X > k.xend_frac)) {
            reflect_split(gxn, X, k.xend_cell, k.xend_frac);
            ux = 2.f * k.u0 - ux; uy = -uy; uz = -uz;
            flip = true;
          }
        }
        if (flip) {
          on[0] = X;
          inc[0] = gxn - ci;
          if (inc[0] < -1 || inc[0] > 1) {
            atomicOr(d.err, EB_MOVED_TOO_FAR);
            inc[0] = max(-1, min(1, inc[0]));
          }
        }
      }
      leaver = (inc[0] | inc[1] | inc[2]) != 0;
      // the slot of the previous leaver has had a whole iteration to return
      if (ppos >= 0) write_pending3(ppos);
      ppos = -1;
      if (leaver) {
        const int nlx = lx + inc[0], nly = ly + inc[1], nlz = lz + inc[2];
        // its new tile among the 3 x 3 x 3 neighbourhood (>> of -1 is -1)
        const int q = ((nlz >> 2) + 1) * 9 + ((nly >> 3) + 1) * 3 + ((nlx >> 3) + 1);
        const int s = sp1 ? 1 : 0;
        const int dlc = ((nlz & (TZ - 1)) * TY + (nly & (TY - 1))) * TX + (nlx & (TX - 1));
        ppos = atomicAdd(&m.acnt[nb_bin[s][q] * TC + dlc], 1);  // used in the next iteration
        pend->w[c][0] = make_float4(on[0], on[1], on[2], ux);
        pend->w[c][1] = make_float4(uy, uz, idlo, idhi);
        pend->key[c] = (dir_group3((inc[2] + 1) * 9 + (inc[1] + 1) * 3 + (inc[0] + 1)) << 16) | kk;
        pend->dst[c] = q | (s << 5) | (dlc << 8);
#pragma unroll
        for (int mm = 0; mm < 3; ++mm) {
          lo_[mm] = o[mm];
          ln_[mm] = on[mm];
          linc[mm] = inc[mm];
        }
        lsp1 = sp1;
      } else {
        float4* so = reinterpret_cast<float4*>((sp1 ? col1 + (size_t)n0 * M3_PL : col0) +
                                               (size_t)(sp1 ? j1 : j0) * M3_PL);
        so[0] = make_float4(on[0], on[1], on[2], ux);
        so[1] = make_float4(uy, uz, idlo, idhi);
        if (sp1) ++j1; else ++j0;
        // ---- Esirkepov deposit of a particle that stays in its cell, into the registers ----
        // support: nodes -1, 0, 1 on every axis; ds from the factored difference
        float s0[3][3], ds[3][3], A[3][3], B[3][3];
#pragma unroll
        for (int mm = 0; mm < 3; ++mm) {
          const float dl = on[mm] - o[mm], sp = o[mm] + on[mm];
          ds[mm][0] = -0.5f * dl * (2.f - sp);
          ds[mm][1] = -dl * (sp - 1.f);
          ds[mm][2] = 0.5f * dl * sp;
#pragma unroll
          for (int e = 0; e < 3; ++e) {
            s0[mm][e] = w[mm][e];
            A[mm][e] = (s0[mm][e] + 0.5f * ds[mm][e]) * qdd;
            B[mm][e] = (0.5f * s0[mm][e] + third * ds[mm][e]) * qdd;
          }
        }
        // own-axis prefixes: edge 0 carries -ds[0], edge 1 carries -(ds[0] + ds[1])
        const float2 px = make_float2(-ds[0][0], -ds[0][0] - ds[0][1]);
        const float2 py = make_float2(-ds[1][0], -ds[1][0] - ds[1][1]);
        const float2 pz = make_float2(-ds[2][0], -ds[2][0] - ds[2][1]);
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
          for (int kq = 0; kq < 3; ++kq) {
            // x: transverse y (j), z (kq); y: x (j), z (kq); z: x (j), y (kq)
            const float tx_ = A[1][j] * s0[2][kq] + B[1][j] * ds[2][kq];
            const float ty_ = A[0][j] * s0[2][kq] + B[0][j] * ds[2][kq];
            const float tz_ = A[0][j] * s0[1][kq] + B[0][j] * ds[1][kq];
            acc.jx[j][kq] = __ffma2_rn(px, make_float2(tx_, tx_), acc.jx[j][kq]);
            acc.jy[j][kq] = __ffma2_rn(py, make_float2(ty_, ty_), acc.jy[j][kq]);
            acc.jz[j][kq] = __ffma2_rn(pz, make_float2(tz_, tz_), acc.jz[j][kq]);
          }
      }
    }
    // leavers join the warp's queue; 32 queued are deposited one per lane
    const unsigned lm = __ballot_sync(0xffffffffu, leaver);
    if (leaver) {
      const int e = (qtail + __popc(lm & ((1u << lane) - 1u))) & (LQ - 1);
      myq[0 * LQ + e] = lo_[0];
      myq[1 * LQ + e] = lo_[1];
      myq[2 * LQ + e] = lo_[2];
      myq[3 * LQ + e] = ln_[0];
      myq[4 * LQ + e] = ln_[1];
      myq[5 * LQ + e] = ln_[2];
      myq[6 * LQ + e] =
          __int_as_float((linc[0] + 1) | ((linc[1] + 1) << 2) | ((linc[2] + 1) << 4) | ((lsp1 ? 1 : 0) << 6) | (c << 8));
    }
    qtail += __popc(lm);
    __syncwarp();
    if (qtail - qhead >= 32) drain(32);
    if ((t & (FLUSH_EVERY - 1)) == FLUSH_EVERY - 1) cell3_flush(acc, jhi, jlo, lx, ly, lz, fs1, fis1, fs2);
    issue(t + PF);
  }
  cp_async_wait<0>();
  if (ppos >= 0) write_pending3(ppos);
  if (qtail > qhead) drain(qtail - qhead);
  m.ccnt[bin0 * TC + c] = j0;
  if (nsp > 1) m.ccnt[(bin0 + 1) * TC + c] = j1;
  if (tw & (FLUSH_EVERY - 1)) cell3_flush(acc, jhi, jlo, lx, ly, lz, fs1, fis1, fs2);
  __syncthreads();
  // one flush of the patch into the global fixed-point current (exact 64-bit integer sums): patch
  // node (xl, yl, zl) is field index (cx0 + xl, cy0 + yl, cz0 + zl); the ghost fold follows
  for (int idx = c; idx < 3 * JN; idx += TC) {
    const int ih = jhi[idx], il = jlo[idx];
    if ((ih | il) == 0) continue;
    const long long v = (long long)ih * 32768LL + (long long)il;
    const int xl = idx % JX, yl = (idx / JX) % JY, zl = (idx / (JX * JY)) % JZ, comp = idx / JN;
    const size_t f = (size_t)(cx0 + xl) + (size_t)g.fp * ((size_t)(cy0 + yl) + (size_t)(g.ny + 4) * (cz0 + zl));
    atomicAdd(&m.ujx[(size_t)comp * g.fvol + f], (unsigned long long)v);
  }
}

void mix3_push(const Dev3D& d, const Mix3Const& k, const void* tmap, bool vay, cudaStream_t s) {
  cudaMemsetAsync(d.m.ujx, 0, sizeof(unsigned long long) * 3 * d.g.fvol, s);
  if (vay)
    k_mix3_push<true><<<d.m.ntile, TC, PUSH_SMEM, s>>>(d, k, *(const CUtensorMap*)tmap);
  else
    k_mix3_push<false><<<d.m.ntile, TC, PUSH_SMEM, s>>>(d, k, *(const CUtensorMap*)tmap);
}

// fixed point -> FP64 current over the whole ghosted extent (the fold of bc__curre follows)
__global__ void k_mix3_fix(Dev3D d) {
  const size_t n = 3 * d.g.fvol;
  const double is2 = d.m.fx_is2;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    d.uj[i] = (double)(long long)d.m.ujx[i] * is2;
}

void mix3_fix(const Dev3D& d, cudaStream_t s) { k_mix3_fix<<<8 * 152, 256, 0, s>>>(d); }

// ---------------------------------------------------------------------------
// arrivals (per bin, thread = destination cell): the push left the cell's j stayers in slots
// 0 .. j-1 and its b arrivals in slots dep-1 down to dep-b; they move to slots j .. j+b-1 in the
// order of their keys (direction of arrival, then slot in the source column).  The kernel also
// records per bin count + 2 x arrivals of its fullest column; past 7/8 of the depth the host
// grows the bin before the next push.
// ---------------------------------------------------------------------------
constexpr int ARR_KR = 8;  // keys per cell held in registers; more are read from global memory
constexpr int ARR_BATCH = 4;

__global__ void __launch_bounds__(TC) k_mix3_arrive(Dev3D d) {
  __shared__ int wmax[TC / 32];
  const Mix3D& m = d.m;
  const int bin = blockIdx.x;
  const int c = threadIdx.x;
  const int dep = m.bdep[bin];
  const int nold = m.cnt[bin * TC + c];
  const int j = m.ccnt[bin * TC + c];
  int b = m.acnt[bin * TC + c];
  bool ok = true;
  if (b > dep || nold + b > dep || j + 2 * b > dep) {
    ok = false;
    atomicOr(d.err, EB_CAPACITY);
  }
  if (b > dep) b = dep;
  const int bm = ok ? b : 0;  // arrivals moved
  float* const col = mix3_slot(m, bin, 0, c);
  const float* top = col + (size_t)(dep - 1) * M3_PL;  // arrival i in slot dep - 1 - i
  const int* ktop = mix3_key(m, bin, dep - 1, c);
  auto key = [&](int i) { return ktop[-(ptrdiff_t)i * TC]; };
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
#pragma unroll
  for (int h = 0; h < ARR_KR; h += ARR_BATCH) {
    int dl[ARR_BATCH];
    float4 w[ARR_BATCH][2];
#pragma unroll
    for (int u = 0; u < ARR_BATCH; ++u) {
      dl[u] = h + u < bm ? j + rank_of(kr[h + u]) : -1;
      if (dl[u] >= 0) {
        const float4* src = reinterpret_cast<const float4*>(top - (size_t)(h + u) * M3_PL);
        w[u][0] = src[0];
        w[u][1] = src[1];
      }
    }
#pragma unroll
    for (int u = 0; u < ARR_BATCH; ++u)
      if (dl[u] >= 0) {
        float4* dst = reinterpret_cast<float4*>(col + (size_t)dl[u] * M3_PL);
        dst[0] = w[u][0];
        dst[1] = w[u][1];
      }
  }
  for (int i = ARR_KR; i < bm; ++i) {
    const int dl = j + rank_of(key(i));
    const float4* src = reinterpret_cast<const float4*>(top - (size_t)i * M3_PL);
    const float4 w0 = src[0], w1 = src[1];
    float4* dst = reinterpret_cast<float4*>(col + (size_t)dl * M3_PL);
    dst[0] = w0;
    dst[1] = w1;
  }
  const int nn = ok ? j + b : j;
  m.cnt[bin * TC + c] = nn;
  m.acnt[bin * TC + c] = 0;
  int need = nn + 2 * b;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) need = max(need, __shfl_xor_sync(0xffffffffu, need, o));
  if ((c & 31) == 0) wmax[c >> 5] = need;
  __syncthreads();
  if (c == 0) {
    for (int w = 1; w < TC / 32; ++w) need = max(need, wmax[w]);
    m.bneed[bin] = need;
    if (8 * (long long)need > 7 * (long long)dep) atomicOr(m.grow, 1);
  }
}

void mix3_arrive(const Dev3D& d, cudaStream_t s) { k_mix3_arrive<<<d.m.nbin, TC, 0, s>>>(d); }

// copy of every column (cnt slots, the eight data planes) from another layout into d.m's
__global__ void __launch_bounds__(TC) k_mix3_relayout(Dev3D d, const float* from_P, const long long* from_boff) {
  const Mix3D& m = d.m;
  const int bin = blockIdx.x, c = threadIdx.x;
  const int n = m.cnt[bin * TC + c];
  const float4* src = reinterpret_cast<const float4*>(from_P + ((size_t)from_boff[bin] * TC + c) * M3_W);
  float4* dst = reinterpret_cast<float4*>(mix3_slot(m, bin, 0, c));
  for (int kk = 0; kk < n; ++kk) {
    const size_t o = (size_t)kk * (M3_PL / 4);
    const float4 a = src[o], b = src[o + 1];
    dst[o] = a;
    dst[o + 1] = b;
  }
}

void mix3_relayout(const Dev3D& d, const float* from_P, const long long* from_boff, cudaStream_t s) {
  k_mix3_relayout<<<d.m.nbin, TC, 0, s>>>(d, from_P, from_boff);
}

int mix3_initial_depth(double n, double c_dt_dx) {
  // count with a 25 % rise and 5 standard deviations of Poisson noise, plus room for the arrivals
  // of the first steps (a particle crosses a face of its cell with probability <= c dt / dx per axis)
  const double cf = c_dt_dx < 1.0 ? c_dt_dx : 1.0;
  const double arr = 0.6 * n * cf + 3.0 * std::sqrt(0.6 * n * cf) + 2.0;
  const double dep = 1.25 * n + 5.0 * std::sqrt(n) + 2.0 * arr + 8.0;
  int kk = ((int)std::ceil(dep) + 7) & ~7;
  return kk > MIX_MAX_DEPTH ? MIX_MAX_DEPTH : kk;
}

// ---------------------------------------------------------------------------
// reference layout <-> columns.  A chunk holds the 4 ny rows of species isp and z layers
// 4 tz .. 4 tz + 3 (row r of the chunk = (kk - 4 tz) ny + jj, np_host slots of ndim words each).
// One CTA per tile of the chunk: for each of its 32 bucket rows the 8 cells' particles are one
// contiguous range of the row (cumcnt); consecutive threads take consecutive words.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(TC) k_mix3_put(Dev3D d, const double* aos, int ndim, int np_host, int isp, int tz) {
  __shared__ int scc[TZ * TY][TX + 1];
  const Mix3D& m = d.m;
  const Grid3D g = d.g;
  const int tx = blockIdx.x, ty = blockIdx.y;
  const int bin = ((tz * m.nty + ty) * m.ntx + tx) * d.ph.nsp + isp;
  const int c = threadIdx.x;
  const int dep = m.bdep[bin];
  for (int t = c; t < TZ * TY * (TX + 1); t += TC) {
    const int r = t / (TX + 1), q = t - r * (TX + 1);  // r = lz * TY + ly
    const int kk = tz * TZ + r / TY, jj = ty * TY + r % TY;
    scc[r][q] = d.cc[((size_t)(isp * g.nz + kk) * g.ny + jj) * (g.nx + 1) + tx * TX + q];
  }
  __syncthreads();
  {
    const int lx = c & (TX - 1), r = c >> 3;
    int n = scc[r][lx + 1] - scc[r][lx];
    if (n > dep) {
      atomicOr(d.err, EB_CAPACITY);
      n = dep;
    }
    m.cnt[bin * TC + c] = n;
  }
  const double dxi = d.ph.d_delx;
  float* const cl0 = mix3_slot(m, bin, 0, 0);
  for (int r = 0; r < TZ * TY; ++r) {
    const int lz = r / TY, ly = r % TY;
    const int kk = tz * TZ + lz, jj = ty * TY + ly;
    const int first = scc[r][0];
    const long long nw = (long long)(scc[r][TX] - first) * ndim;
    const double* rowp = aos + ((size_t)(lz * g.ny + jj) * np_host + first) * ndim;
    for (long long w = c; w < nw; w += TC) {
      const int pl = (int)(w / ndim), comp = (int)(w - (long long)pl * ndim);
      const int p = first + pl;
      int lx = 0;
#pragma unroll
      for (int step = 4; step > 0; step >>= 1)
        if (scc[r][lx + step] <= p) lx += step;
      const int kq = p - scc[r][lx];
      if (kq >= dep || comp > 6) continue;
      const double a = rowp[w];
      float* o = cl0 + (size_t)kq * M3_PL + (r * TX + lx) * M3_W;
      const int gx = tx * TX + lx;
      // offsets in [0, 1): a position within 2^-25 cells below a face rounds up to 1 in FP32
      if (comp == 0) o[M3_OX] = fminf((float)(a * dxi - (double)(g.nxgs + gx)), 0.99999994f);
      else if (comp == 1) o[M3_OY] = fminf((float)(a * dxi - (double)(g.nygs + jj)), 0.99999994f);
      else if (comp == 2) o[M3_OZ] = fminf((float)(a * dxi - (double)(g.nzgs + kk)), 0.99999994f);
      else if (comp == 3) o[M3_UX] = (float)a;
      else if (comp == 4) o[M3_UY] = (float)a;
      else if (comp == 5) o[M3_UZ] = (float)a;
      else {
        const long long id = __double_as_longlong(a);
        o[M3_IDLO] = __int_as_float((int)(unsigned)(id & 0xffffffffll));
        o[M3_IDHI] = __int_as_float((int)(unsigned)((unsigned long long)id >> 32));
      }
    }
  }
}

void mix3_put(const Dev3D& d, const double* aos, int ndim, int np_host, int isp, int tz, cudaStream_t s) {
  k_mix3_put<<<dim3(d.m.ntx, d.m.nty), TC, 0, s>>>(d, aos, ndim, np_host, isp, tz);
}

// per bin, the largest particle count of its cells in the reference-layout cumcnt (d.cc)
__global__ void __launch_bounds__(TC) k_mix3_binmax(Dev3D d) {
  __shared__ int wmax[TC / 32];
  const Mix3D& m = d.m;
  const Grid3D g = d.g;
  const int bin = blockIdx.x;
  const int nsp = d.ph.nsp;
  const int tile = bin / nsp, isp = bin - tile * nsp;
  const int tx = tile % m.ntx, ty = (tile / m.ntx) % m.nty, tz = tile / (m.ntx * m.nty);
  const int c = threadIdx.x;
  const int gx = tx * TX + (c & (TX - 1)), jj = ty * TY + ((c >> 3) & (TY - 1)), kk = tz * TZ + (c >> 6);
  const int* ccr = d.cc + ((size_t)(isp * g.nz + kk) * g.ny + jj) * (g.nx + 1);
  int v = ccr[gx + 1] - ccr[gx];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((c & 31) == 0) wmax[c >> 5] = v;
  __syncthreads();
  if (c == 0) {
    for (int w = 1; w < TC / 32; ++w) v = max(v, wmax[w]);
    m.bneed[bin] = v;
  }
}

void mix3_binmax(const Dev3D& d, cudaStream_t s) { k_mix3_binmax<<<d.m.nbin, TC, 0, s>>>(d); }

// columns -> reference layout: per row an exclusive scan of the column counts into cumcnt and np2
__global__ void __launch_bounds__(32) k_mix3_rowscan(Dev3D d) {
  const Mix3D& m = d.m;
  const Grid3D g = d.g;
  const int row = blockIdx.x;  // (isp * nz + kk) * ny + jj
  const int jj = row % g.ny, kk = (row / g.ny) % g.nz, isp = row / (g.ny * g.nz);
  const int lane = threadIdx.x;
  const int nx = g.nx;
  int* ccr = d.cc + (size_t)row * (nx + 1);
  const int ty = jj / TY, tz = kk / TZ;
  const int cbase = ((kk % TZ) * TY + jj % TY) * TX;
  int carry = 0;
  for (int k0 = 0; k0 < nx; k0 += 32) {
    const int gx = k0 + lane;
    int v = 0;
    if (gx < nx) {
      const int bin = ((tz * m.nty + ty) * m.ntx + gx / TX) * d.ph.nsp + isp;
      v = m.cnt[bin * TC + cbase + gx % TX];
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

void mix3_count_rows(const Dev3D& d, cudaStream_t s) { k_mix3_rowscan<<<d.nrow, 32, 0, s>>>(d); }

// the reverse of k_mix3_put: the tile's particles of each bucket row written as one contiguous
// AoS range (cumcnt from k_mix3_rowscan), cell by cell in column order
__global__ void __launch_bounds__(TC) k_mix3_get(Dev3D d, double* aos, int ndim, int np_host, int isp, int tz) {
  __shared__ int scc[TZ * TY][TX + 1];
  const Mix3D& m = d.m;
  const Grid3D g = d.g;
  const int tx = blockIdx.x, ty = blockIdx.y;
  const int bin = ((tz * m.nty + ty) * m.ntx + tx) * d.ph.nsp + isp;
  const int c = threadIdx.x;
  for (int t = c; t < TZ * TY * (TX + 1); t += TC) {
    const int r = t / (TX + 1), q = t - r * (TX + 1);
    const int kk = tz * TZ + r / TY, jj = ty * TY + r % TY;
    scc[r][q] = d.cc[((size_t)(isp * g.nz + kk) * g.ny + jj) * (g.nx + 1) + tx * TX + q];
  }
  __syncthreads();
  const double dx = d.ph.delx;
  const float* const cl0 = mix3_slot(m, bin, 0, 0);
  for (int r = 0; r < TZ * TY; ++r) {
    const int lz = r / TY, ly = r % TY;
    const int kk = tz * TZ + lz, jj = ty * TY + ly;
    const int first = scc[r][0];
    int last = scc[r][TX];
    if (last > np_host) {
      if (c == 0) atomicOr(d.err, EB_CAPACITY);
      last = np_host;
    }
    const long long nw = (long long)(last - first) * ndim;
    double* rowp = aos + ((size_t)(lz * g.ny + jj) * np_host + (first > 0 ? first : 0)) * ndim;
    for (long long w = c; w < nw; w += TC) {
      const int pl = (int)(w / ndim), comp = (int)(w - (long long)pl * ndim);
      const int p = first + pl;
      int lx = 0;
#pragma unroll
      for (int step = 4; step > 0; step >>= 1)
        if (scc[r][lx + step] <= p) lx += step;
      const int kq = p - scc[r][lx];
      const float* o = cl0 + (size_t)kq * M3_PL + (r * TX + lx) * M3_W;
      const int gx = tx * TX + lx;
      double v;
      if (comp == 0) v = ((double)(g.nxgs + gx) + (double)o[M3_OX]) * dx;
      else if (comp == 1) v = ((double)(g.nygs + jj) + (double)o[M3_OY]) * dx;
      else if (comp == 2) v = ((double)(g.nzgs + kk) + (double)o[M3_OZ]) * dx;
      else if (comp == 3) v = (double)o[M3_UX];
      else if (comp == 4) v = (double)o[M3_UY];
      else if (comp == 5) v = (double)o[M3_UZ];
      else if (comp == 6) {
        const unsigned long long id = ((unsigned long long)(unsigned)__float_as_int(o[M3_IDHI]) << 32) |
                                      (unsigned)__float_as_int(o[M3_IDLO]);
        v = __longlong_as_double((long long)id);
      } else {
        v = 0.0;
      }
      rowp[w] = v;
    }
  }
}

void mix3_get(const Dev3D& d, double* aos, int ndim, int np_host, int isp, int tz, cudaStream_t s) {
  k_mix3_get<<<dim3(d.m.ntx, d.m.nty), TC, 0, s>>>(d, aos, ndim, np_host, isp, tz);
}

// ---------------------------------------------------------------------------
// device loader: the plasma of k_load_weibel3d (same Philox counters: row-local particle index
// k = cx ppc + kk, row rs = kk_z ny + jj); copy kk of cell c goes to slot (kk, c)
// ---------------------------------------------------------------------------
__global__ void k_mix3_load(Dev3D d, int ppc, unsigned long long seed, double drift, int axis, double u_thi,
                            double u_the) {
  const Mix3D& m = d.m;
  const Grid3D g = d.g;
  const int bin = blockIdx.x;
  const int nsp = d.ph.nsp;
  const int tile = bin / nsp, isp = bin - tile * nsp;
  const int tx = tile % m.ntx, ty = (tile / m.ntx) % m.nty, tz = tile / (m.ntx * m.nty);
  const int s = blockIdx.y * blockDim.x + threadIdx.x;  // = kk * 256 + c
  const int c = s % TC, kq = s / TC;
  const int dep = m.bdep[bin];
  if (kq == 0) m.cnt[bin * TC + c] = ppc < dep ? ppc : dep;
  if (kq >= ppc || kq >= dep) return;
  const int cx = tx * TX + (c & (TX - 1)), jj = ty * TY + ((c >> 3) & (TY - 1)), kz = tz * TZ + (c >> 6);
  const int rs = kz * g.ny + jj;
  const int kp = cx * ppc + kq;
  const int npr = g.nx * ppc;
  const uint2 key = make_uint2((unsigned)seed, (unsigned)(seed >> 32));
  const uint4 rp = philox4x32(make_uint4((unsigned)kp, (unsigned)rs, 0u, 0u), key);
  const uint4 rz = philox4x32(make_uint4((unsigned)kp, (unsigned)rs, 7u, 0u), key);
  const uint4 r1 = philox4x32(make_uint4((unsigned)kp, (unsigned)rs, 1u + 2u * isp, 0u), key);
  const uint4 r2 = philox4x32(make_uint4((unsigned)kp, (unsigned)rs, 2u + 2u * isp, 0u), key);
  auto frac = [](double u) {
    const float f = (float)(floor((1.0 - u) * 1099511627776.0) * (1.0 / 1099511627776.0));
    return f < 1.f ? f : 0.99999994f;
  };
  float* const o = mix3_slot(m, bin, kq, c);
  o[M3_OX] = frac(u01(rp.x, rp.y));
  o[M3_OY] = frac(u01(rp.z, rp.w));
  o[M3_OZ] = frac(u01(rz.x, rz.y));
  const double sd = isp == 0 ? u_thi : u_the;
  const double twopi = 6.283185307179586;
  const double a1 = u01(r1.x, r1.y), b1 = u01(r1.z, r1.w), a2 = u01(r2.x, r2.y), b2 = u01(r2.z, r2.w);
  const double rad1 = sqrt(-2.0 * log(a1)), rad2 = sqrt(-2.0 * log(a2));
  double u[3] = {sd * rad1 * cos(twopi * b1), sd * rad1 * sin(twopi * b1), sd * rad2 * cos(twopi * b2)};
  if (isp == 1 && drift != 0.0) u[axis] += (kp % 2 == 0) ? drift : -drift;
  o[M3_UX] = (float)u[0];
  o[M3_UY] = (float)u[1];
  o[M3_UZ] = (float)u[2];
  const long long id = -((long long)rs * npr + kp + 1);
  o[M3_IDLO] = __int_as_float((int)(unsigned)(id & 0xffffffffll));
  o[M3_IDHI] = __int_as_float((int)(unsigned)((unsigned long long)id >> 32));
}

void mix3_load_weibel(const Dev3D& d, int ppc, unsigned long long seed, double drift, int drift_axis, double u_thi,
                      double u_the, cudaStream_t s) {
  dim3 grid(d.m.nbin, (TC * ppc + 255) / 256);  // bins on x: more than 65535 of them at 256^3
  k_mix3_load<<<grid, 256, 0, s>>>(d, ppc, seed, drift, drift_axis, u_thi, u_the);
}

// kinetic energy sums in FP64 over the FP32 momenta (3d/proj/weibel/app.f90:531-552)
__global__ void __launch_bounds__(TC) k_mix3_energy(Dev3D d) {
  __shared__ double sh[TC];
  const Mix3D& m = d.m;
  const int isp = blockIdx.y;
  const double c = d.ph.c, rr = d.ph.r[isp];
  double v = 0.0;
  for (int tile = blockIdx.x; tile < m.ntile; tile += gridDim.x) {
    const int bin = tile * d.ph.nsp + isp;
    const int n = m.cnt[bin * TC + threadIdx.x];
    const float* col = mix3_slot(m, bin, 0, threadIdx.x);
    for (int kq = 0; kq < n; ++kq) {
      const float* o = col + (size_t)kq * M3_PL;
      const double a = o[M3_UX], b = o[M3_UY], e = o[M3_UZ];
      v += rr * (sqrt(1.0 + (a * a + b * b + e * e) / (c * c)) - 1.0);
    }
  }
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int w = TC / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) d.partials[((size_t)isp * d.nred + blockIdx.x) * 2] = sh[0];
}

void mix3_energy(const Dev3D& d, cudaStream_t s) {
  cudaMemsetAsync(d.partials, 0, sizeof(double) * 2 * 3 * (size_t)d.nred, s);
  const int nb = d.nred < d.m.ntile ? d.nred : d.m.ntile;
  k_mix3_energy<<<dim3(nb, d.ph.nsp), TC, 0, s>>>(d);
  fast::energy_fields_fin3d(d, s);
}

// ---------------------------------------------------------------------------
// mom_calc__accl + mom_calc__nvt (3d/common/mom_calc.f90:49-332) on the columns: the half-step
// push (time step halved by mom_calc__init, :36) in FP32, then the seven moments of each particle
// at its 2 x 2 x 2 half-integer nodes (node index floor(x/dx - 0.5): cell - 1 or cell), summed in
// the tile's 10 x 10 x 6 node patch with FP32 shared atomics and added once per node into the
// FP64 moments.  The state is not modified.
// ---------------------------------------------------------------------------
constexpr int MX = TX + 2, MY = TY + 2, MZ = TZ + 2;  // nodes at cell offsets -1 .. T

__global__ void __launch_bounds__(TC) k_mix3_mom(Dev3D d, Mix3Const k, double* mom) {
  __shared__ float tf[6][FZ][FY][FX];
  __shared__ float macc[7][MZ][MY][MX];
  const Mix3D& m = d.m;
  const Grid3D g = d.g;
  const int tile = blockIdx.x, isp = blockIdx.y;
  const int tx = tile % m.ntx, ty = (tile / m.ntx) % m.nty, tz = tile / (m.ntx * m.nty);
  const int cx0 = tx * TX, cy0 = ty * TY, cz0 = tz * TZ;
  const int t = threadIdx.x;
  for (int idx = t; idx < FN; idx += TC) {
    const int a = idx % FX, bb = (idx / FX) % FY, cc = idx / (FX * FY);
    const size_t f = (size_t)(cx0 + a + 1) + (size_t)g.fp * ((size_t)(cy0 + bb + 1) + (size_t)(g.ny + 4) * (cz0 + cc + 1));
    const size_t V = g.fvol, I = 1, J = g.fp, K = g.fplane;
    const double* U = d.uf;
    tf[0][cc][bb][a] = (float)(2.5e-1 * (U[f] + U[f + J] + U[f + K] + U[f + J + K]));
    tf[1][cc][bb][a] = (float)(2.5e-1 * (U[V + f] + U[V + f + I] + U[V + f + K] + U[V + f + I + K]));
    tf[2][cc][bb][a] = (float)(2.5e-1 * (U[2 * V + f] + U[2 * V + f + I] + U[2 * V + f + J] + U[2 * V + f + I + J]));
    tf[3][cc][bb][a] = (float)(5e-1 * (U[3 * V + f] + U[3 * V + f + I]));
    tf[4][cc][bb][a] = (float)(5e-1 * (U[4 * V + f] + U[4 * V + f + J]));
    tf[5][cc][bb][a] = (float)(5e-1 * (U[5 * V + f] + U[5 * V + f + K]));
  }
  for (int idx = t; idx < 7 * MX * MY * MZ; idx += TC) (&macc[0][0][0][0])[idx] = 0.f;
  __syncthreads();
  const int lx = t & (TX - 1), ly = (t >> 3) & (TY - 1), lz = t >> 6;
  const float cl = k.c, ic2 = k.ic2;
  const float fac1 = 0.5f * k.fac1[isp], fac2 = 0.5f * k.fac2[isp];  // half time step
  const float txxx = fac1 * fac1;
  const int bin = tile * d.ph.nsp + isp;
  const int n = m.cnt[bin * TC + t];
  const float* col = mix3_slot(m, bin, 0, t);
  for (int s = 0; s < n; ++s) {
    const float* pp = col + (size_t)s * M3_PL;
    const float o[3] = {pp[M3_OX], pp[M3_OY], pp[M3_OZ]};
    float w[3][3];
#pragma unroll
    for (int mm = 0; mm < 3; ++mm) {
      w[mm][0] = 0.5f * (1.f - o[mm]) * (1.f - o[mm]);
      w[mm][1] = 0.75f - (o[mm] - 0.5f) * (o[mm] - 0.5f);
      w[mm][2] = 0.5f * o[mm] * o[mm];
    }
    float f[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int c3 = 0; c3 < 3; ++c3)
#pragma unroll
      for (int b3 = 0; b3 < 3; ++b3) {
        const float wzy = w[2][c3] * w[1][b3];
#pragma unroll
        for (int a3 = 0; a3 < 3; ++a3) {
          const float wt = wzy * w[0][a3];
#pragma unroll
          for (int mm = 0; mm < 6; ++mm) f[mm] = fmaf(wt, tf[mm][lz + c3][ly + b3][lx + a3], f[mm]);
        }
      }
    const float bpx = f[0], bpy = f[1], bpz = f[2], epx = f[3], epy = f[4], epz = f[5];
    float u1 = pp[M3_UX] + fac1 * epx, u2 = pp[M3_UY] + fac1 * epy, u3 = pp[M3_UZ] + fac1 * epz;
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
    const float pre[7] = {1.f, ux * gam, uy * gam, uz * gam, ux * ux * gam, uy * uy * gam, uz * uz * gam};
    float wl[3][2];
    int nb[3];
#pragma unroll
    for (int mm = 0; mm < 3; ++mm) {
      const float h = o[mm] - 0.5f;
      nb[mm] = h < 0.f ? 0 : 1;
      const float dd = h < 0.f ? h + 1.f : h;
      wl[mm][0] = 1.f - dd;
      wl[mm][1] = dd;
    }
#pragma unroll
    for (int cz = 0; cz < 2; ++cz)
#pragma unroll
      for (int by = 0; by < 2; ++by)
#pragma unroll
        for (int ax = 0; ax < 2; ++ax) {
          const float wt = wl[0][ax] * wl[1][by] * wl[2][cz];
          const int xl = lx + nb[0] + ax, yl = ly + nb[1] + by, zl = lz + nb[2] + cz;
#pragma unroll
          for (int l = 0; l < 7; ++l) atomicAdd(&macc[l][zl][yl][xl], pre[l] * wt);
        }
  }
  __syncthreads();
  // the patch into the FP64 moments of this species: local node (xl, yl, zl) is node index
  // (cx0 + xl, cy0 + yl, cz0 + zl) of mom(7, nxgs-1:nxge+1, nys-1:nye+1, nzs-1:nze+1, nsp)
  const size_t nxm = g.nx + 2, nym = g.ny + 2, nzm = g.nz + 2;
  for (int idx = t; idx < MX * MY * MZ; idx += TC) {
    const int xl = idx % MX, yl = (idx / MX) % MY, zl = idx / (MX * MY);
    double* out = mom + 7 * ((size_t)(cx0 + xl) + nxm * ((size_t)(cy0 + yl) + nym * ((size_t)(cz0 + zl) + nzm * isp)));
#pragma unroll
    for (int l = 0; l < 7; ++l) {
      const float v = macc[l][zl][yl][xl];
      if (v != 0.f) atomicAdd(out + l, (double)v);
    }
  }
}

void mix3_moments(const Dev3D& d, const Mix3Const& k, double* mom, cudaStream_t s) {
  cudaMemsetAsync(mom, 0, sizeof(double) * 7 * (size_t)(d.g.nx + 2) * (d.g.ny + 2) * (d.g.nz + 2) * d.ph.nsp, s);
  k_mix3_mom<<<dim3(d.m.ntile, d.ph.nsp), TC, 0, s>>>(d, k, mom);
  bc_mom3d(d, mom, s);
}

bool mix3_shape_ok(int nx, int ny, int nz) { return nx % TX == 0 && ny % TY == 0 && nz % TZ == 0; }

int mix3_setup(const Dev3D& d, void* out) {
  typedef CUresult (*EncodeFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                               const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                               CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn)
    return -1;
  // uf as [6][nz+4][ny+4][nx+4] FP64; the box starts at an even column (16-byte rule for x)
  const cuuint64_t dims[4] = {(cuuint64_t)d.g.fp, (cuuint64_t)(d.g.ny + 4), (cuuint64_t)(d.g.nz + 4), 6};
  const cuuint64_t strides[3] = {(cuuint64_t)d.g.fp * sizeof(double), (cuuint64_t)d.g.fplane * sizeof(double),
                                 (cuuint64_t)d.g.fvol * sizeof(double)};
  const cuuint32_t box[4] = {SX, SY, SZ, 6};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = ((EncodeFn)fn)((CUtensorMap*)out, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, d.uf, dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return -2;
  if (cudaFuncSetAttribute(k_mix3_push<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, PUSH_SMEM) != cudaSuccess ||
      cudaFuncSetAttribute(k_mix3_push<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, PUSH_SMEM) != cudaSuccess)
    return -3;
  return 0;
}

}  // namespace wpic
