// Mixed-precision 3D path: FP32 push, gather and Esirkepov deposition on split positions
// (integer cell + FP32 offset), FP32 currents summed exactly in fixed point and converted
// to FP64 global J; FP64 field state, solver and particle bookkeeping (the 3D FP64 kernels).
//
// One CTA of 256 threads per 8 x 8 x 4-cell tile runs particle__solv and ele_cur fused
// (3d/common/particle.f90:52-233, 3d/common/field.f90:211-406); thread c walks the
// particles of cell c (both species) in the row-bucket layout of the FP64 path:
//  * the tile's cell-centred E/B (10 x 10 x 6 cells x 6 components) is formed once in
//    shared memory in FP32 from the FP64 fields;
//  * each particle's offset in its cell is taken in FP32, pushed (Buneman-Boris in
//    Gaussian units), moved, and written back as cell + FP32 offset (exact in FP64);
//  * its Esirkepov current (the reference's factored form, FP32, the spline difference
//    in the factored form that keeps small displacements accurate) goes into the tile's
//    current patch (12 x 12 x 8 nodes x 3 components) as exact two-plane fixed point with
//    32-bit shared-memory integer atomics, and the patch is added once into a global int64
//    fixed-point current, converted to FP64 J by k_mix3_fix.
// The particle state stays in the FP64 layout (x, y, z, ux, uy, uz, id) so that the
// boundary, migration, sort, moment and exchange kernels of the FP64 path apply unchanged;
// its values are those of the split representation.
#include <cmath>

#include "common.cuh"
#include "mixed_common.cuh"

namespace wpic {

namespace {

constexpr int T3X = 8, T3Y = 8, T3Z = 4;
constexpr int T3C = T3X * T3Y * T3Z;                   // threads = cells per tile
constexpr int F3X = T3X + 2, F3Y = T3Y + 2, F3Z = T3Z + 2;  // centred fields of cells -1 .. T
constexpr int J3X = T3X + 4, J3Y = T3Y + 4, J3Z = T3Z + 4;  // current nodes at offsets -2 .. T + 1
constexpr int LO_PLANE_LIMIT = 100000;  // particles per tile that the low fixed-point plane can sum
constexpr int PF3 = 4;                  // particles in flight per thread (shared-memory ring)
constexpr int RING_BYTES = PF3 * 7 * T3C * 8;

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ size_t fidx3(const Grid3D& g, int fi, int fj, int fk) {
  return (size_t)fi + (size_t)g.fp * ((size_t)fj + (size_t)(g.ny + 4) * (size_t)fk);
}

// p = old offset + displacement (cell units, |displacement| < 1): new cell increment and
// offset in [0, 1).  A step a hair below the lower face, where p + 1 rounds to 1, keeps
// the particle at offset 0 of its old cell.
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

}  // namespace

// VAY: the push of particle__solv_vay (3d/common/particle.f90:236-419) in place of the
// Buneman-Boris rotation; gather, move and deposit are the same.
template <bool VAY>
__global__ void __launch_bounds__(T3C, 2) k_mix3_step(Dev3D d, Mix3Const k, long long* ujx) {
  __shared__ float tf[6][F3Z][F3Y][F3X];
  __shared__ int jhi[3][J3Z][J3Y][J3X];
  __shared__ int jlo[3][J3Z][J3Y][J3X];
  __shared__ int npop;
  const Grid3D g = d.g;
  const int ntx = g.nx / T3X, nty = g.ny / T3Y;
  const int b = blockIdx.x;
  const int cx0 = (b % ntx) * T3X, cy0 = ((b / ntx) % nty) * T3Y, cz0 = (b / (ntx * nty)) * T3Z;
  const int t = threadIdx.x;
  // cell-centred fields (3d/common/particle.f90:75-92): local cell (a-1, bb-1, cc-1) has
  // field index (cx0 + a + 1, cy0 + bb + 1, cz0 + cc + 1)
  for (int idx = t; idx < F3X * F3Y * F3Z; idx += T3C) {
    const int a = idx % F3X, bb = (idx / F3X) % F3Y, cc = idx / (F3X * F3Y);
    const size_t f = fidx3(g, cx0 + a + 1, cy0 + bb + 1, cz0 + cc + 1);
    const size_t V = g.fvol, I = 1, J = g.fp, K = g.fplane;
    const double* U = d.uf;
    tf[0][cc][bb][a] = (float)(2.5e-1 * (U[f] + U[f + J] + U[f + K] + U[f + J + K]));
    tf[1][cc][bb][a] = (float)(2.5e-1 * (U[V + f] + U[V + f + I] + U[V + f + K] + U[V + f + I + K]));
    tf[2][cc][bb][a] = (float)(2.5e-1 * (U[2 * V + f] + U[2 * V + f + I] + U[2 * V + f + J] + U[2 * V + f + I + J]));
    tf[3][cc][bb][a] = (float)(5e-1 * (U[3 * V + f] + U[3 * V + f + I]));
    tf[4][cc][bb][a] = (float)(5e-1 * (U[4 * V + f] + U[4 * V + f + J]));
    tf[5][cc][bb][a] = (float)(5e-1 * (U[5 * V + f] + U[5 * V + f + K]));
  }
  for (int idx = t; idx < 3 * J3X * J3Y * J3Z; idx += T3C) {
    (&jhi[0][0][0][0])[idx] = 0;
    (&jlo[0][0][0][0])[idx] = 0;
  }
  if (t == 0) npop = 0;
  __syncthreads();
  const int lx = t % T3X, ly = (t / T3X) % T3Y, lz = t / (T3X * T3Y);
  const int ci = cx0 + lx, cj = cy0 + ly, ck = cz0 + lz;
  int mine = 0;
  for (int isp = 0; isp < d.ph.nsp; ++isp) {
    const int* ccr = d.cc + (size_t)((isp * g.nz + ck) * g.ny + cj) * (g.nx + 1);
    mine += ccr[ci + 1] - ccr[ci];
  }
  atomicAdd(&npop, mine);
  __syncthreads();
  const int ntile = npop;
  if (ntile == 0) return;  // uniform across the CTA
  if (ntile > LO_PLANE_LIMIT) {
    if (t == 0) atomicOr(d.err, EB_CAPACITY);
    return;
  }
  // tile scale: |v s1| < 2^22 per contribution and every node's sum of hi below 2^30
  const int E1 = min(k.eA, ilogbf(1073741824.f / ((float)ntile * k.vmax)));
  const float s1 = ldexpf(1.f, E1), is1 = ldexpf(1.f, -E1), s2 = ldexpf(1.f, E1 + 15);

  const double dxi = d.ph.p_d_delx, dx = d.ph.delx;
  const int ia = g.nxgs + ci, ja = g.nygs + cj, ka = g.nzgs + ck;
  const float dtdx = k.dtdx, cl = k.c, ic2 = k.ic2, third = 1.0f / 3.0f;
  // the cell's particles, species 0 then species 1, stream through a per-thread ring of PF3
  // slots in shared memory (cp.async), so that PF3 particle loads per thread are in flight
  extern __shared__ __align__(16) double ring[];  // [PF3][7][T3C]
  const int nsp = d.ph.nsp;
  const int row0 = ck * g.ny + cj, row1 = (g.nz + ck) * g.ny + cj;
  const int* cc0 = d.cc + (size_t)row0 * (g.nx + 1);
  const int sb0 = cc0[ci], n0 = cc0[ci + 1] - sb0;
  int sb1 = 0, n1 = 0;
  if (nsp > 1) {
    const int* cc1 = d.cc + (size_t)row1 * (g.nx + 1);
    sb1 = cc1[ci];
    n1 = cc1[ci + 1] - sb1;
  }
  const int ntot = n0 + n1;
  const size_t q0 = (size_t)row0 * d.cap + sb0, q1 = (size_t)row1 * d.cap + sb1 - n0;
  const double* const src[7] = {d.A.x, d.A.y, d.A.z, d.A.ux, d.A.uy, d.A.uz,
                                reinterpret_cast<const double*>(d.A.id)};
  auto issue = [&](int it) {
    if (it < ntot) {
      const size_t q = (it < n0 ? q0 : q1) + it;
      double* dst = ring + (size_t)(it & (PF3 - 1)) * 7 * T3C + t;
#pragma unroll
      for (int a = 0; a < 7; ++a) cp_async8(dst + a * T3C, src[a] + q);
    }
    cp_commit();
  };
#pragma unroll
  for (int it = 0; it < PF3; ++it) issue(it);
  for (int it = 0; it < ntot; ++it) {
    cp_wait<PF3 - 1>();
    const bool sp1 = it >= n0;
    const size_t q = (sp1 ? q1 : q0) + it;
    const double* pb = ring + (size_t)(it & (PF3 - 1)) * 7 * T3C + t;
    const double X = pb[0], Y = pb[T3C], Z = pb[2 * T3C];
    const float ux0 = (float)pb[3 * T3C], uy0 = (float)pb[4 * T3C], uz0 = (float)pb[5 * T3C];
    const long long pid = __double_as_longlong(pb[6 * T3C]);
    const float fac1 = sp1 ? k.fac1[1] : k.fac1[0];
    const float fac2 = sp1 ? k.fac2[1] : k.fac2[0];
    const float qdd = sp1 ? k.qdd[1] : k.qdd[0];
    const float txxx = fac1 * fac1;
    float o[3] = {(float)(X * dxi - (double)ia), (float)(Y * dxi - (double)ja), (float)(Z * dxi - (double)ka)};
    float w[3][3];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      o[m] = fminf(fmaxf(o[m], 0.f), 0.99999994f);
      w[m][0] = 0.5f * (1.f - o[m]) * (1.f - o[m]);
      w[m][1] = 0.75f - (o[m] - 0.5f) * (o[m] - 0.5f);
      w[m][2] = 0.5f * o[m] * o[m];
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
          for (int m = 0; m < 6; ++m) f[m] = fmaf(wt, tf[m][lz + c3][ly + b3][lx + a3], f[m]);
        }
      }
    const float bpx = f[0], bpy = f[1], bpz = f[2], epx = f[3], epy = f[4], epz = f[5];
    float ux, uy, uz, ig;
    if constexpr (VAY) {
      // Vay: gamma of the old momentum, the full electric kick plus the half rotation, then
      // the implicit rotation solved in closed form; the move uses that solution's gamma
      const float fac1r = fac1 * rsqrtf(cl * cl + ux0 * ux0 + uy0 * uy0 + uz0 * uz0);
      const float u4 = ux0 + fac2 * epx + fac1r * (uy0 * bpz - uz0 * bpy);
      const float u5 = uy0 + fac2 * epy + fac1r * (uz0 * bpx - ux0 * bpz);
      const float u6 = uz0 + fac2 * epz + fac1r * (ux0 * bpy - uy0 * bpx);
      const float icl = ic2 * cl;
      const float tx = fac1 * bpx * icl, ty = fac1 * bpy * icl, tz = fac1 * bpz * icl;
      const float tau2 = tx * tx + ty * ty + tz * tz;
      const float ua = (u4 * tx + u5 * ty + u6 * tz) * icl;
      const float sigma = 1.f + (u4 * u4 + u5 * u5 + u6 * u6) * ic2 - tau2;
      const float gam2 = 0.5f * (sigma + sqrtf(sigma * sigma + 4.f * (tau2 + ua * ua)));
      ig = rsqrtf(gam2);
      const float gv = gam2 * ig;
      const float t = __fdividef(1.f, tau2 + gam2);
      ux = t * (gam2 * u4 + cl * ua * tx + gv * (u5 * tz - u6 * ty));
      uy = t * (gam2 * u5 + cl * ua * ty + gv * (u6 * tx - u4 * tz));
      uz = t * (gam2 * u6 + cl * ua * tz + gv * (u4 * ty - u5 * tx));
    } else {
      // Buneman-Boris (3d/common/particle.f90:182-205)
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
    if (d.ph.bc != BC_PERIODIC) {
      // the x boundary before the deposit, in the drivers' order.  Reconnection: particle_x
      // (3d/proj/reconnection/app.f90:103-108), reflection about the walls at cells 1 and
      // nx-2 of the grid (nxs+1 and nxe-1), all three momentum components reversed
      // (3d/proj/reconnection/boundary_reconnection.f90:69-101).  Shock: boundary_shock__injection
      // (3d/proj/shock/app.f90:112-113, boundary_shock.f90:424-469), reflection about cell wx0 + 1
      // of the window with the momenta reversed, and beyond xend x -> 2 xend - x,
      // u_x -> 2 u0 - u_x, u_y and u_z reversed.
      const int gxn = ci + inc[0];
      float X = (float)gxn + on[0];
      bool flip = false;
      if (d.ph.bc == BC_RECONNECTION) {
        if (gxn < 1) { X = 2.f - X; flip = true; }
        else if (gxn >= g.nx - 2) { X = 2.f * (float)(g.nx - 2) - X; flip = true; }
        if (flip) { ux = -ux; uy = -uy; uz = -uz; }
      } else {
        if (gxn < g.wx0 + 1) {
          X = 2.f * (float)(g.wx0 + 1) - X;
          ux = -ux; uy = -uy; uz = -uz;
          flip = true;
        } else if (X > k.xend) {
          X = 2.f * k.xend - X;
          ux = 2.f * k.u0 - ux; uy = -uy; uz = -uz;
          flip = true;
        }
      }
      if (flip) {
        const float fX = floorf(X);
        on[0] = X - fX;
        inc[0] = (int)fX - ci;
        if (on[0] >= 1.f) { on[0] = 0.f; inc[0] += 1; }
        if (inc[0] < -1 || inc[0] > 1) {
          atomicOr(d.err, EB_MOVED_TOO_FAR);
          inc[0] = max(-1, min(1, inc[0]));
        }
      }
    }
    d.B.x[q] = ((double)(ia + inc[0]) + (double)on[0]) * dx;
    d.B.y[q] = ((double)(ja + inc[1]) + (double)on[1]) * dx;
    d.B.z[q] = ((double)(ka + inc[2]) + (double)on[2]) * dx;
    d.B.ux[q] = (double)ux;
    d.B.uy[q] = (double)uy;
    d.B.uz[q] = (double)uz;
    d.B.id[q] = pid;
    // Esirkepov deposit (3d/common/field.f90:331-381).  Along every axis the support of s0 and
    // s1 is 3 nodes (4 when the particle changes cell), starting at node offset lo - 2; the
    // spline arrays are taken in that 4-node window (s0w, dsw).  Along the component's own
    // axis the current is the prefix -sum(ds) dstmp, nonzero on the width - 1 edges inside the
    // support; across it the factor dstmp of the reference.
    float s0w[3][4], dsw[3][4], pre[3][3];
    int lo[3], wd[3];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      float s0[5] = {0.f, w[m][0], w[m][1], w[m][2], 0.f}, ds[5];
      shape_diff5(o[m], on[m], inc[m], ds);
      lo[m] = inc[m] < 0 ? 0 : 1;          // window start: node offset lo - 2
      wd[m] = inc[m] != 0 ? 4 : 3;         // support width
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
      const int t1 = comp == 0 ? 1 : 0;  // transverse axes: t1 (jw) and t2 (kw)
      const int t2 = comp == 2 ? 1 : 2;
      // node = cell + (window offset) along each axis; local patch coordinate = l + lo + i + ...
      const int ea = (comp == 0 ? lx : comp == 1 ? ly : lz) + lo[comp] + 1;  // own axis, edge i at ea + i
      const int e1 = (t1 == 0 ? lx : ly) + lo[t1];
      const int e2 = (t2 == 1 ? ly : lz) + lo[t2];
#pragma unroll
      for (int kw = 0; kw < 4; ++kw) {
        if (kw >= wd[t2]) continue;
#pragma unroll
        for (int jw = 0; jw < 4; ++jw) {
          if (jw >= wd[t1]) continue;
          const float dstmp = ((s0w[t1][jw] + 0.5f * dsw[t1][jw]) * s0w[t2][kw] +
                               (0.5f * s0w[t1][jw] + third * dsw[t1][jw]) * dsw[t2][kw]) * qdd;
#pragma unroll
          for (int aw = 0; aw < 3; ++aw) {
            if (aw >= wd[comp] - 1) continue;
            int xl, yl, zl;
            if (comp == 0) { xl = ea + aw; yl = e1 + jw; zl = e2 + kw; }
            else if (comp == 1) { xl = e1 + jw; yl = ea + aw; zl = e2 + kw; }
            else { xl = e1 + jw; yl = e2 + kw; zl = ea + aw; }
            fx_add(&jhi[comp][zl][yl][xl], &jlo[comp][zl][yl][xl], pre[comp][aw] * dstmp, s1, is1, s2);
          }
        }
      }
    }
    issue(it + PF3);
  }
  cp_wait<0>();
  __syncthreads();
  // the patch into the global fixed point (scale 2^G): node (xl, yl, zl) has field index
  // (cx0 + xl, cy0 + yl, cz0 + zl)
  const int shift = k.G - (E1 + 15);
  for (int idx = t; idx < 3 * J3X * J3Y * J3Z; idx += T3C) {
    const int xl = idx % J3X, yl = (idx / J3X) % J3Y, zl = (idx / (J3X * J3Y)) % J3Z, comp = idx / (J3X * J3Y * J3Z);
    const int h = (&jhi[0][0][0][0])[idx], l = (&jlo[0][0][0][0])[idx];
    if ((h | l) == 0) continue;
    long long v = (long long)h * 32768 + (long long)l;
    v = shift >= 0 ? (v << shift) : (v >> (-shift));
    atomicAdd(reinterpret_cast<unsigned long long*>(ujx + (size_t)comp * g.fvol + fidx3(g, cx0 + xl, cy0 + yl, cz0 + zl)),
              (unsigned long long)v);
  }
}

// uj = ujx 2^-G over the whole ghosted array; ujx cleared for the next step
__global__ void k_mix3_fix(Dev3D d, long long* ujx, double scale) {
  const size_t n = 3 * d.g.fvol;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    d.uj[i] = (double)ujx[i] * scale;
    ujx[i] = 0;
  }
}

void mix3_push_deposit(const Dev3D& d, const Mix3Const& k, long long* ujx, bool vay, cudaStream_t s) {
  const int ntile = (d.g.nx / T3X) * (d.g.ny / T3Y) * (d.g.nz / T3Z);
  if (vay)
    k_mix3_step<true><<<ntile, T3C, RING_BYTES, s>>>(d, k, ujx);
  else
    k_mix3_step<false><<<ntile, T3C, RING_BYTES, s>>>(d, k, ujx);
  k_mix3_fix<<<4 * 152, 256, 0, s>>>(d, ujx, std::ldexp(1.0, -k.G));
}

// ---------------------------------------------------------------------------
// mom_calc__accl + mom_calc__nvt (3d/common/mom_calc.f90:49-332) for the mixed path: the
// half-step push (time step halved by mom_calc__init, :36) in FP32 on split positions, then
// the seven moments of each particle at its 2 x 2 x 2 half-integer nodes (node index
// floor(x/dx - 0.5), cell - 1 or cell), summed in the tile's 10 x 10 x 6 node patch with FP32
// shared atomics and added once per node into the FP64 moments.  The state is not modified.
// ---------------------------------------------------------------------------
constexpr int M3X = T3X + 2, M3Y = T3Y + 2, M3Z = T3Z + 2;  // nodes at cell offsets -1 .. T

__global__ void __launch_bounds__(T3C, 2) k_mix3_mom(Dev3D d, Mix3Const k, double* mom) {
  __shared__ float tf[6][F3Z][F3Y][F3X];
  __shared__ float macc[7][M3Z][M3Y][M3X];
  const Grid3D g = d.g;
  const int ntx = g.nx / T3X, nty = g.ny / T3Y;
  const int b = blockIdx.x;
  const int cx0 = (b % ntx) * T3X, cy0 = ((b / ntx) % nty) * T3Y, cz0 = (b / (ntx * nty)) * T3Z;
  const int t = threadIdx.x;
  for (int idx = t; idx < F3X * F3Y * F3Z; idx += T3C) {
    const int a = idx % F3X, bb = (idx / F3X) % F3Y, cc = idx / (F3X * F3Y);
    const size_t f = fidx3(g, cx0 + a + 1, cy0 + bb + 1, cz0 + cc + 1);
    const size_t V = g.fvol, I = 1, J = g.fp, K = g.fplane;
    const double* U = d.uf;
    tf[0][cc][bb][a] = (float)(2.5e-1 * (U[f] + U[f + J] + U[f + K] + U[f + J + K]));
    tf[1][cc][bb][a] = (float)(2.5e-1 * (U[V + f] + U[V + f + I] + U[V + f + K] + U[V + f + I + K]));
    tf[2][cc][bb][a] = (float)(2.5e-1 * (U[2 * V + f] + U[2 * V + f + I] + U[2 * V + f + J] + U[2 * V + f + I + J]));
    tf[3][cc][bb][a] = (float)(5e-1 * (U[3 * V + f] + U[3 * V + f + I]));
    tf[4][cc][bb][a] = (float)(5e-1 * (U[4 * V + f] + U[4 * V + f + J]));
    tf[5][cc][bb][a] = (float)(5e-1 * (U[5 * V + f] + U[5 * V + f + K]));
  }
  for (int idx = t; idx < 7 * M3X * M3Y * M3Z; idx += T3C) (&macc[0][0][0][0])[idx] = 0.f;
  __syncthreads();
  const int lx = t % T3X, ly = (t / T3X) % T3Y, lz = t / (T3X * T3Y);
  const int ci = cx0 + lx, cj = cy0 + ly, ck = cz0 + lz;
  const double dxi = d.ph.p_d_delx;
  const int ia = g.nxgs + ci, ja = g.nygs + cj, ka = g.nzgs + ck;
  const float cl = k.c, ic2 = k.ic2;
  for (int isp = 0; isp < d.ph.nsp; ++isp) {
    const int row = (isp * g.nz + ck) * g.ny + cj;
    const int* ccr = d.cc + (size_t)row * (g.nx + 1);
    const int sb = ccr[ci], se = ccr[ci + 1];
    const float fac1 = 0.5f * k.fac1[isp], fac2 = 0.5f * k.fac2[isp];  // half time step
    const float txxx = fac1 * fac1;
    const size_t rbase = (size_t)row * d.cap;
    for (int s = sb; s < se; ++s) {
      const size_t q = rbase + s;
      float o[3] = {(float)(d.A.x[q] * dxi - (double)ia), (float)(d.A.y[q] * dxi - (double)ja),
                    (float)(d.A.z[q] * dxi - (double)ka)};
      float w[3][3];
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        o[m] = fminf(fmaxf(o[m], 0.f), 0.99999994f);
        w[m][0] = 0.5f * (1.f - o[m]) * (1.f - o[m]);
        w[m][1] = 0.75f - (o[m] - 0.5f) * (o[m] - 0.5f);
        w[m][2] = 0.5f * o[m] * o[m];
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
            for (int m = 0; m < 6; ++m) f[m] = fmaf(wt, tf[m][lz + c3][ly + b3][lx + a3], f[m]);
          }
        }
      const float bpx = f[0], bpy = f[1], bpz = f[2], epx = f[3], epy = f[4], epz = f[5];
      float u1 = (float)d.A.ux[q] + fac1 * epx, u2 = (float)d.A.uy[q] + fac1 * epy, u3 = (float)d.A.uz[q] + fac1 * epz;
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
      // node index cell - 1 (offset < 1/2) or cell; local node coordinate = l + (0 or 1)
      float wl[3][2];
      int nb[3];
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        const float h = o[m] - 0.5f;
        nb[m] = h < 0.f ? 0 : 1;
        const float dd = h < 0.f ? h + 1.f : h;
        wl[m][0] = 1.f - dd;
        wl[m][1] = dd;
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
    for (int idx = t; idx < M3X * M3Y * M3Z; idx += T3C) {
      const int xl = idx % M3X, yl = (idx / M3X) % M3Y, zl = idx / (M3X * M3Y);
      double* out = mom + 7 * ((size_t)(cx0 + xl) +
                               nxm * ((size_t)(cy0 + yl) + nym * ((size_t)(cz0 + zl) + nzm * isp)));
#pragma unroll
      for (int l = 0; l < 7; ++l) {
        const float v = macc[l][zl][yl][xl];
        if (v != 0.f) atomicAdd(out + l, (double)v);
        macc[l][zl][yl][xl] = 0.f;
      }
    }
    __syncthreads();
  }
}

void mix3_moments(const Dev3D& d, const Mix3Const& k, double* mom, cudaStream_t s) {
  const int ntile = (d.g.nx / T3X) * (d.g.ny / T3Y) * (d.g.nz / T3Z);
  cudaMemsetAsync(mom, 0, sizeof(double) * 7 * (size_t)(d.g.nx + 2) * (d.g.ny + 2) * (d.g.nz + 2) * d.ph.nsp, s);
  k_mix3_mom<<<ntile, T3C, 0, s>>>(d, k, mom);
  bc_mom3d(d, mom, s);
}

bool mix3_shape_ok(int nx, int ny, int nz) { return nx % T3X == 0 && ny % T3Y == 0 && nz % T3Z == 0; }

int mix3_setup() {
  return cudaFuncSetAttribute(k_mix3_step<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, RING_BYTES) ==
                     cudaSuccess &&
                 cudaFuncSetAttribute(k_mix3_step<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, RING_BYTES) ==
                     cudaSuccess
             ? 0
             : -1;
}

}  // namespace wpic
