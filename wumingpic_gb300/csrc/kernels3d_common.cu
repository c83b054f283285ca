// Precision-independent kernels of the 3D FP64 path: current and field ghost
// rules (3d/common/boundary_periodic.f90), particle boundaries (x wrap and the
// (y, z) migration), the stable bucket sort, layout conversions and the device
// loader.  Integer work here is bit-exact against the reference.
#include <algorithm>

#include "common.cuh"

namespace wpic {

namespace {

__device__ __forceinline__ size_t g3(const Grid3D& g, int fi, int fj, int fk) {
  return (size_t)fi + (size_t)g.fp * ((size_t)fj + (size_t)(g.ny + 4) * (size_t)fk);
}

}  // namespace

// ---------------------------------------------------------------------------
// boundary_periodic__curre  (3d/common/boundary_periodic.f90:676-978), one rank.
// Each stage is one kernel so that the reference's statement order holds:
//   y fold over k = nzs-2..nze+2 (ghost rows nys-2, nys-1 added into nye-1, nye;
//   then nye+1, nye+2 into nys, nys+1), z fold over j = nys..nye, the 1-deep
//   margins (y for k = nzs..nze, then z for j = nys-1..nye+1), then the x fold
//   and x refresh over everything.  Requires nx, ny, nz >= 4 (checked at init),
//   so that no statement reads a value another statement of the same stage writes.
// ---------------------------------------------------------------------------
__global__ void k_curre3d_y(Dev3D d) {  // thread per (fi, fk), all ghosted
  const Grid3D g = d.g;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.fp * (g.nz + 4)) return;
  const int fi = t % g.fp, fk = t / g.fp;
  const int ny = g.ny;
  for (int l = 0; l < 3; ++l) {
    double* u = d.uj + (size_t)l * g.fvol;
    const double a0 = u[g3(g, fi, 0, fk)], a1 = u[g3(g, fi, 1, fk)];
    u[g3(g, fi, ny, fk)] = u[g3(g, fi, ny, fk)] + a0;          // nye-1 += nys-2
    u[g3(g, fi, ny + 1, fk)] = u[g3(g, fi, ny + 1, fk)] + a1;  // nye   += nys-1
    const double b0 = u[g3(g, fi, ny + 2, fk)], b1 = u[g3(g, fi, ny + 3, fk)];
    u[g3(g, fi, 2, fk)] = u[g3(g, fi, 2, fk)] + b0;  // nys   += nye+1
    u[g3(g, fi, 3, fk)] = u[g3(g, fi, 3, fk)] + b1;  // nys+1 += nye+2
  }
}

__global__ void k_curre3d_z(Dev3D d) {  // thread per (fi, j interior)
  const Grid3D g = d.g;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.fp * g.ny) return;
  const int fi = t % g.fp, fj = t / g.fp + 2;
  const int nz = g.nz;
  for (int l = 0; l < 3; ++l) {
    double* u = d.uj + (size_t)l * g.fvol;
    const double a0 = u[g3(g, fi, fj, 0)], a1 = u[g3(g, fi, fj, 1)];
    u[g3(g, fi, fj, nz)] = u[g3(g, fi, fj, nz)] + a0;
    u[g3(g, fi, fj, nz + 1)] = u[g3(g, fi, fj, nz + 1)] + a1;
    const double b0 = u[g3(g, fi, fj, nz + 2)], b1 = u[g3(g, fi, fj, nz + 3)];
    u[g3(g, fi, fj, 2)] = u[g3(g, fi, fj, 2)] + b0;
    u[g3(g, fi, fj, 3)] = u[g3(g, fi, fj, 3)] + b1;
  }
}

__global__ void k_curre3d_margin_y(Dev3D d) {  // thread per (fi, k interior): nye+1 <- nys, nys-1 <- nye
  const Grid3D g = d.g;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.fp * g.nz) return;
  const int fi = t % g.fp, fk = t / g.fp + 2;
  for (int l = 0; l < 3; ++l) {
    double* u = d.uj + (size_t)l * g.fvol;
    u[g3(g, fi, g.ny + 2, fk)] = u[g3(g, fi, 2, fk)];
    u[g3(g, fi, 1, fk)] = u[g3(g, fi, g.ny + 1, fk)];
  }
}

__global__ void k_curre3d_margin_z(Dev3D d) {  // thread per (fi, j = nys-1..nye+1): nze+1 <- nzs, nzs-1 <- nze
  const Grid3D g = d.g;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.fp * (g.ny + 2)) return;
  const int fi = t % g.fp, fj = t / g.fp + 1;
  for (int l = 0; l < 3; ++l) {
    double* u = d.uj + (size_t)l * g.fvol;
    u[g3(g, fi, fj, g.nz + 2)] = u[g3(g, fi, fj, 2)];
    u[g3(g, fi, fj, 1)] = u[g3(g, fi, fj, g.nz + 1)];
  }
}

__global__ void k_curre3d_x(Dev3D d) {  // thread per (fj, fk), all ghosted
  const Grid3D g = d.g;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (g.ny + 4) * (g.nz + 4)) return;
  const int fj = t % (g.ny + 4), fk = t / (g.ny + 4);
  const int nx = g.nx;
  for (int l = 0; l < 3; ++l) {
    double* u = d.uj + (size_t)l * g.fvol + g3(g, 0, fj, fk);
    u[nx] = u[nx] + u[0];
    u[nx + 1] = u[nx + 1] + u[1];
    u[2] = u[2] + u[nx + 2];
    u[3] = u[3] + u[nx + 3];
    u[0] = u[nx];
    u[1] = u[nx + 1];
    u[nx + 2] = u[2];
    u[nx + 3] = u[3];
  }
}

void curre_fold3d(const Dev3D& d, cudaStream_t s) {
  const Grid3D& g = d.g;
  k_curre3d_y<<<(g.fp * (g.nz + 4) + 127) / 128, 128, 0, s>>>(d);
  k_curre3d_z<<<(g.fp * g.ny + 127) / 128, 128, 0, s>>>(d);
  k_curre3d_margin_y<<<(g.fp * g.nz + 127) / 128, 128, 0, s>>>(d);
  k_curre3d_margin_z<<<(g.fp * (g.ny + 2) + 127) / 128, 128, 0, s>>>(d);
  // boundary_reconnection__curre has no x stage (3d/proj/reconnection/boundary_reconnection.f90:689-978)
  if (d.ph.bc == BC_PERIODIC) k_curre3d_x<<<((g.ny + 4) * (g.nz + 4) + 127) / 128, 128, 0, s>>>(d);
}

// ---------------------------------------------------------------------------
// boundary_periodic__dfield (3d/common/boundary_periodic.f90:458-673): the copies y, z, x
// leave every ghost of the 2-deep halo equal to its periodic image (nx, ny, nz >= 2)
// ---------------------------------------------------------------------------
__global__ void k_dfield3d(Dev3D d) {
  const Grid3D g = d.g;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < g.fvol; t += (size_t)gridDim.x * blockDim.x) {
    const int fi = (int)(t % g.fp), fj = (int)((t / g.fp) % (g.ny + 4)), fk = (int)(t / g.fplane);
    const bool ghost = fi < 2 || fi >= g.nx + 2 || fj < 2 || fj >= g.ny + 2 || fk < 2 || fk >= g.nz + 2;
    if (!ghost) continue;
    int si = fi - 2, sj = fj - 2, sk = fk - 2;
    si = si < 0 ? si + g.nx : (si >= g.nx ? si - g.nx : si);
    sj = sj < 0 ? sj + g.ny : (sj >= g.ny ? sj - g.ny : sj);
    sk = sk < 0 ? sk + g.nz : (sk >= g.nz ? sk - g.nz : sk);
    const size_t src = g3(g, si + 2, sj + 2, sk + 2);
    for (int l = 0; l < 6; ++l) d.df[(size_t)l * g.fvol + t] = d.df[(size_t)l * g.fvol + src];
  }
}

// boundary_reconnection__dfield (3d/proj/reconnection/boundary_reconnection.f90:466-686): the
// periodic y and z copies over the interior x columns, then at the walls, for every (j, k)
// including the ghosts, Bx and (Ey, Ez) odd -- column nxs-1 from nxs, column nxe (an interior
// column) from nxe-1 -- and (By, Bz, Ex) even -- nxs-1 from nxs+1, nxe+1 from nxe-1; columns
// nxs-2 and nxe+2 are left as they are.  Every value read is an interior-x value the rule does
// not write, so one pass over the cells is the reference's sequence.
// boundary_shock__dfield (3d/proj/shock/boundary_shock.f90:472-687) differs only at the right
// end: every component zero in column nxe+1, column nxe kept.  Both act on the window
// nxs..nxe (array columns wx0+2 .. wx1+2); the y and z copies cover the window's columns.
__global__ void k_dfield3d_walls(Dev3D d) {
  const Grid3D g = d.g;
  const bool shock = d.ph.bc == BC_SHOCK;
  const int cs = g.wx0 + 2, ce = g.wx1 + 2;  // array columns of nxs and nxe
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < g.fvol; t += (size_t)gridDim.x * blockDim.x) {
    const int fi = (int)(t % g.fp), fj = (int)((t / g.fp) % (g.ny + 4)), fk = (int)(t / g.fplane);
    const bool yz_ghost = fj < 2 || fj >= g.ny + 2 || fk < 2 || fk >= g.nz + 2;
    int sj = fj - 2, sk = fk - 2;
    sj = sj < 0 ? sj + g.ny : (sj >= g.ny ? sj - g.ny : sj);
    sk = sk < 0 ? sk + g.nz : (sk >= g.nz ? sk - g.nz : sk);
    auto src = [&](int l, int si) { return d.df[(size_t)l * g.fvol + g3(g, si, sj + 2, sk + 2)]; };
    for (int l = 0; l < 6; ++l) {
      const bool odd = l == 0 || l == 4 || l == 5;
      double* out = d.df + (size_t)l * g.fvol + t;
      if (fi == cs - 1) *out = odd ? -src(l, cs) : src(l, cs + 1);
      else if (shock && fi == ce + 1) *out = 0.0;
      else if (!shock && fi == ce && odd) *out = -src(l, ce - 1);
      else if (!shock && fi == ce + 1 && !odd) *out = src(l, ce - 1);
      else if (fi >= cs && fi <= ce && yz_ghost) *out = src(l, fi);
    }
  }
}

void dfield_ghost3d(const Dev3D& d, cudaStream_t s) {
  if (d.ph.bc == BC_PERIODIC) k_dfield3d<<<8 * 152, 256, 0, s>>>(d);
  else k_dfield3d_walls<<<8 * 152, 256, 0, s>>>(d);
}

// uf += df over the whole ghosted extent (3d/common/field.f90:196-205)
__global__ void k_uf_add3d(Dev3D d) {
  const size_t n = 6 * d.g.fvol;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    d.uf[t] = d.uf[t] + d.df[t];
}

void uf_add3d(const Dev3D& d, cudaStream_t s) { k_uf_add3d<<<8 * 152, 256, 0, s>>>(d); }

// ---------------------------------------------------------------------------
// boundary_periodic__particle_x  (3d/common/boundary_periodic.f90:68-101), default rounding
// ---------------------------------------------------------------------------
__global__ void k_particle_x3d(Dev3D d, Parts3D P) {  // one block per row
  const int row = blockIdx.x;
  const Grid3D g = d.g;
  const int nxge = g.nxgs + g.nx - 1;
  const int n = d.np2[row];
  for (int s = threadIdx.x; s < n; s += blockDim.x) {
    const size_t k = (size_t)row * d.cap + s;
    double x = P.x[k];
    const int ipos = (int)(x * d.ph.p_d_delx);
    if (ipos < g.nxgs) x = x + (double)g.nx * d.ph.delx;
    else if (ipos >= nxge + 1) x = x - (double)g.nx * d.ph.delx;
    P.x[k] = x;
  }
}

// boundary_reconnection__particle_x (3d/proj/reconnection/boundary_reconnection.f90:69-109): cell
// int(x / dx) below nxs+1 or from nxe-1 on reflects about that face, 2 (nxs+1) dx - x or
// 2 (nxe-1) dx - x, all three momentum components reversed; separately rounded as the reference
__global__ void k_particle_x3d_walls(Dev3D d, Parts3D P) {  // one block per row
  const int row = blockIdx.x;
  const Grid3D g = d.g;
  const int nxs = g.nxgs, nxe = g.nxgs + g.nx - 1;
  const double delx = d.ph.delx;
  const int n = d.np2[row];
  for (int s = threadIdx.x; s < n; s += blockDim.x) {
    const size_t k = (size_t)row * d.cap + s;
    const double x = P.x[k];
    const int ipos = (int)__ddiv_rn(x, delx);
    double face;
    if (ipos < nxs + 1) face = __dmul_rn(2.0 * (nxs + 1), delx);
    else if (ipos >= nxe - 1) face = __dmul_rn(2.0 * (nxe - 1), delx);
    else continue;
    P.x[k] = __dsub_rn(face, x);
    P.ux[k] = -P.ux[k];
    P.uy[k] = -P.uy[k];
    P.uz[k] = -P.uz[k];
  }
}

// boundary_shock__injection (3d/proj/shock/boundary_shock.f90:424-469): cell int(x / dx) (the
// product with 1/dx) below nxs+1 reflects about (nxs+1) dx with all momenta reversed; beyond
// xend (computed on the host) x -> 2 xend - x, u_x -> 2 u0 - u_x, u_y and u_z reversed
__global__ void k_injection3d(Dev3D d, Parts3D P, double u0, double xend) {  // one block per row
  const int row = blockIdx.x;
  const int nxs = d.g.nxgs + d.g.wx0;
  const double delx = d.ph.delx;
  const int n = d.np2[row];
  for (int s = threadIdx.x; s < n; s += blockDim.x) {
    const size_t k = (size_t)row * d.cap + s;
    const double x = P.x[k];
    const int ipos = (int)__dmul_rn(x, d.ph.p_d_delx);
    if (ipos < nxs + 1) {
      P.x[k] = __dsub_rn(__dmul_rn(2.0 * (nxs + 1), delx), x);
      P.ux[k] = -P.ux[k];
      P.uy[k] = -P.uy[k];
      P.uz[k] = -P.uz[k];
    } else if (x > xend) {
      P.x[k] = __dsub_rn(__dmul_rn(2.0, xend), x);
      P.ux[k] = __dsub_rn(__dmul_rn(2.0, u0), P.ux[k]);
      P.uy[k] = -P.uy[k];
      P.uz[k] = -P.uz[k];
    }
  }
}

void injection3d(const Dev3D& d, const Parts3D& P, double u0, double xend, cudaStream_t s) {
  k_injection3d<<<d.nrow, 256, 0, s>>>(d, P, u0, xend);
}

void particle_x3d(const Dev3D& d, const Parts3D& P, cudaStream_t s) {
  if (d.ph.bc == BC_PERIODIC) k_particle_x3d<<<d.nrow, 256, 0, s>>>(d, P);
  else k_particle_x3d_walls<<<d.nrow, 256, 0, s>>>(d, P);
}

// ---------------------------------------------------------------------------
// boundary_periodic__particle_yz (3d/common/boundary_periodic.f90:104-455), first phase:
// per row, each particle's destination (jpos, kpos) = (int(y/dx), int(z/dx)) (the product
// with d_delx, as the reference); a mover is wrapped in y and z and tagged with its direction
// (dy, dz); the row's movers are listed by direction group (0..7, the codes 0..8 without 4),
// slot order inside a group.  One CTA per row.
// ---------------------------------------------------------------------------
constexpr int MIG3_THREADS = 256;

__device__ __forceinline__ int dgroup(int code) { return code < 4 ? code : code - 1; }

__global__ void __launch_bounds__(MIG3_THREADS) k_migrate3d_scan(Dev3D d, Parts3D P) {
  const Grid3D g = d.g;
  const int row = blockIdx.x;
  const int jj = row % g.ny, kk = (row / g.ny) % g.nz;
  const int j = g.nygs + jj, k = g.nzgs + kk;
  const int nyge = g.nygs + g.ny - 1, nzge = g.nzgs + g.nz - 1;
  const int n = d.np2[row];
  const size_t rb = (size_t)row * d.cap;
  const double dxi = d.ph.p_d_delx, delx = d.ph.delx;
  __shared__ int wc[MIG3_THREADS / 32][8];
  __shared__ int base[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // pass 1: wrap, tag, count per group
  if (threadIdx.x < 8) base[threadIdx.x] = 0;
  __syncthreads();
  for (int c0 = 0; c0 < n; c0 += MIG3_THREADS) {
    const int s = c0 + threadIdx.x;
    int code = 4;
    if (s < n) {
      double y = P.y[rb + s], z = P.z[rb + s];
      const int jpos = (int)(y * dxi), kpos = (int)(z * dxi);
      if (!(jpos == j && kpos == k)) {
        const int dy = jpos - j, dz = kpos - k;
        if (dy < -1 || dy > 1 || dz < -1 || dz > 1) {
          atomicOr(d.err, EB_MOVED_TOO_FAR);
        } else {
          code = (dz + 1) * 3 + (dy + 1);
          if (jpos <= g.nygs - 1) y = y + (double)g.ny * delx;
          else if (jpos >= nyge + 1) y = y - (double)g.ny * delx;
          if (kpos <= g.nzgs - 1) z = z + (double)g.nz * delx;
          else if (kpos >= nzge + 1) z = z - (double)g.nz * delx;
          P.y[rb + s] = y;
          P.z[rb + s] = z;
        }
      }
      d.mig[rb + s] = (int8_t)(code == 4 ? 0 : code + 1);
    }
    const int grp = code == 4 ? -1 : dgroup(code);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const unsigned b = __ballot_sync(0xffffffffu, grp == q);
      if (lane == 0) atomicAdd(&base[q], __popc(b));
    }
  }
  __syncthreads();
  int* gcnt = d.gcnt + (size_t)row * 8;
  int* goff = d.goff + (size_t)row * 8;
  __shared__ int off[8];
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int q = 0; q < 8; ++q) {
      gcnt[q] = base[q];
      goff[q] = acc;
      off[q] = acc;
      acc += base[q];
    }
  }
  __syncthreads();
  // pass 2: stable scatter of the movers into their group's range of glist
  for (int c0 = 0; c0 < n; c0 += MIG3_THREADS) {
    const int s = c0 + threadIdx.x;
    int grp = -1;
    if (s < n) {
      const int m = d.mig[rb + s];
      grp = m == 0 ? -1 : dgroup(m - 1);
    }
    unsigned bal[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      bal[q] = __ballot_sync(0xffffffffu, grp == q);
      if (lane == 0) wc[warp][q] = __popc(bal[q]);
    }
    __syncthreads();
    if (grp >= 0) {
      int o = off[grp];
      for (int w = 0; w < warp; ++w) o += wc[w][grp];
      unsigned b = 0;
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (q == grp) b = bal[q];
      d.glist[rb + o + __popc(b & lanemask_lt())] = s;
    }
    __syncthreads();
    if (threadIdx.x < 8)
      for (int w = 0; w < MIG3_THREADS / 32; ++w) off[threadIdx.x] += wc[w][threadIdx.x];
    __syncthreads();
  }
}

void migrate_scan3d(const Dev3D& d, const Parts3D& P, cudaStream_t s) {
  k_migrate3d_scan<<<d.nrow, MIG3_THREADS, 0, s>>>(d, P);
}

// ---------------------------------------------------------------------------
// Second phase: the post-migration slot order of every row in closed form.  The
// arrivals of a row, in the order the reference's buffers hold them (one rank, one
// thread), are these segments -- each the movers of one source row with one direction,
// in slot order:
//  S1 direct: sources (j-dy, k-dz) inside the domain, in the reference's row loop order
//     (k outer, j inner), i.e. dz = +1, 0, -1 and inside each dy = +1, 0, -1;
//  S2 (j = nye): the ghost row (nys-1, k) -- sources (nys, k-dz), dy = -1, dz = +1, 0, -1;
//  S3 (j = nys): the ghost row (nye+1, k) -- sources (nye, k-dz), dy = +1;
//  S4 (k = nze): the ghost row (j, nzs-1) after the y transfers -- its direct sources
//     (j-dy, nzs), dz = -1, dy = +1, 0, -1; then, if j = nye, (nys, nzs) with (dy, dz) =
//     (-1, -1); then, if j = nys, (nye, nzs) with (+1, -1);
//  S5 (k = nzs): the ghost row (j, nze+1) likewise with dz = +1.
// Holes are filled as in the 2D path: b >= h: hole m <- arrival m, slot n+k <- arrival h+k;
// b < h: hole m < b <- arrival m, the remaining holes below n' = n-(h-b) <- the non-hole
// slots of [n', n) in descending order.  One warp per row.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(32) k_migrate3d_plan(Dev3D d) {
  const Grid3D g = d.g;
  const int row = blockIdx.x;
  const int nrs = g.ny * g.nz;
  const int isp = row / nrs;
  const int jj = row % g.ny, kk = (row / g.ny) % g.nz;
  const int lane = threadIdx.x;
  const size_t cap = d.cap;
  const int ny = g.ny, nz = g.nz;
  // segment list: source row, direction group, count, first index in the source's glist
  int srow[24], sgrp[24], scnt[24];
  int ns = 0;
  auto add = [&](int sj, int sk, int dy, int dz) {
    if (sj < 0 || sj >= ny || sk < 0 || sk >= nz) return;
    const int r = (isp * nz + sk) * ny + sj;
    const int q = dgroup((dz + 1) * 3 + (dy + 1));
    srow[ns] = r;
    sgrp[ns] = q;
    scnt[ns] = d.gcnt[(size_t)r * 8 + q];
    ++ns;
  };
  // S1
  for (int dz = 1; dz >= -1; --dz)
    for (int dy = 1; dy >= -1; --dy)
      if (dy != 0 || dz != 0) add(jj - dy, kk - dz, dy, dz);
  // S2, S3
  if (jj == ny - 1)
    for (int dz = 1; dz >= -1; --dz) add(0, kk - dz, -1, dz);
  if (jj == 0)
    for (int dz = 1; dz >= -1; --dz) add(ny - 1, kk - dz, +1, dz);
  // S4, S5
  if (kk == nz - 1) {
    for (int dy = 1; dy >= -1; --dy) add(jj - dy, 0, dy, -1);
    if (jj == ny - 1) add(0, 0, -1, -1);
    if (jj == 0) add(ny - 1, 0, +1, -1);
  }
  if (kk == 0) {
    for (int dy = 1; dy >= -1; --dy) add(jj - dy, nz - 1, dy, +1);
    if (jj == ny - 1) add(0, nz - 1, -1, +1);
    if (jj == 0) add(ny - 1, nz - 1, +1, +1);
  }
  int b = 0;
  for (int t = 0; t < ns; ++t) b += scnt[t];
  const int n = d.np2[row];
  int h = 0;
  for (int q = 0; q < 8; ++q) h += d.gcnt[(size_t)row * 8 + q];
  int nn = n - h + b;
  if (nn > (int)cap) {
    if (lane == 0) atomicOr(d.err, EB_CAPACITY);
    nn = (int)cap;
  }
  if (lane == 0) d.np2new[row] = nn;
  const size_t rb = (size_t)row * cap;
  const unsigned lt = lanemask_lt();
  if (b < h) {
    int kq = 0;
    for (int t0 = n - 1; t0 >= nn; t0 -= 32) {
      const int t = t0 - lane;
      const bool st = t >= nn && d.mig[rb + t] == 0;
      const unsigned bal = __ballot_sync(0xffffffffu, st);
      if (st) d.tlist[rb + kq + __popc(bal & lt)] = t;
      kq += __popc(bal);
    }
  }
  __syncwarp();
  int m0 = 0;
  for (int t0 = 0; t0 < nn; t0 += 32) {
    const int t = t0 + lane;
    const bool act = t < nn;
    const bool hole = act && t < n && d.mig[rb + t] != 0;
    const unsigned hb = __ballot_sync(0xffffffffu, hole);
    const int m = m0 + __popc(hb & lt);
    if (act) {
      int src = 0;
      int a = -1;
      if (t >= n) a = h + (t - n);
      else if (!hole) src = (int)(rb + t);
      else if (m < b) a = m;
      else src = (int)(rb + d.tlist[rb + (m - b)]);
      if (a >= 0) {
        int sg = 0;
        while (a >= scnt[sg]) {
          a -= scnt[sg];
          ++sg;
        }
        const int r = srow[sg];
        const int first = d.goff[(size_t)r * 8 + sgrp[sg]];
        src = (int)((size_t)r * cap + d.glist[(size_t)r * cap + first + a]);
      }
      d.slist[rb + t] = src;
    }
    m0 += __popc(hb);
  }
}

void migrate_plan3d(const Dev3D& d, cudaStream_t s) { k_migrate3d_plan<<<d.nrow, 32, 0, s>>>(d); }

// ---------------------------------------------------------------------------
// sort__bucket (3d/common/sort.f90:40-88): stable counting sort of each row by i = int(x),
// one warp per row, as in the 2D path.  map[pos] = source slot.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(32) k_sort3d_rank(Dev3D d, Parts3D P, const int* slist, const int* counts) {
  extern __shared__ int off3[];
  const Grid3D g = d.g;
  const int row = blockIdx.x;
  const int lane = threadIdx.x;
  const int n = counts[row];
  const int nx = g.nx;
  const size_t rb = (size_t)row * d.cap;
  for (int k = lane; k <= nx; k += 32) off3[k] = 0;
  __syncwarp();
  for (int t0 = 0; t0 < n; t0 += 32) {
    const int t = t0 + lane;
    if (t < n) {
      const int src = slist ? slist[rb + t] : (int)(rb + t);
      int cell = (int)P.x[src] - g.nxgs;
      if (cell < 0 || cell >= nx) {
        atomicOr(d.err, EB_OUT_OF_RANGE);
        cell = cell < 0 ? 0 : nx - 1;
      }
      atomicAdd(&off3[cell], 1);
    }
  }
  __syncwarp();
  int* ccr = d.cc + (size_t)row * (nx + 1);
  int carry = 0;
  for (int k0 = 0; k0 < nx; k0 += 32) {
    const int k = k0 + lane;
    const int v = k < nx ? off3[k] : 0;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const int excl = incl - v + carry;
    if (k < nx) {
      off3[k] = excl;
      ccr[k] = excl;
    }
    carry += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (lane == 0) ccr[nx] = carry;
  __syncwarp();
  const unsigned lt = lanemask_lt();
  for (int t0 = 0; t0 < n; t0 += 32) {
    const int t = t0 + lane;
    const bool act = t < n;
    int src = 0, cell = -1 - lane;
    if (act) {
      src = slist ? slist[rb + t] : (int)(rb + t);
      cell = (int)P.x[src] - g.nxgs;
      cell = cell < 0 ? 0 : (cell >= nx ? nx - 1 : cell);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, cell);
    int base = 0;
    if (act) base = off3[cell];
    __syncwarp();
    if (act && lane == __ffs(peers) - 1) off3[cell] = base + __popc(peers);
    __syncwarp();
    if (act) d.map[rb + base + __popc(peers & lt)] = src;
  }
}

void sort_rank3d(const Dev3D& d, const Parts3D& P, const int* slist, cudaStream_t s) {
  const int* counts = slist ? d.np2new : d.np2;
  k_sort3d_rank<<<d.nrow, 32, (d.g.nx + 1) * sizeof(int), s>>>(d, P, slist, counts);
}

__global__ void k_gather3d(Dev3D d, Parts3D S, Parts3D D, const int* map, const int* counts) {  // block per row
  const int row = blockIdx.x;
  const int n = counts[row];
  for (int pos = threadIdx.x; pos < n; pos += blockDim.x) {
    const size_t k = (size_t)row * d.cap + pos;
    const size_t m = (size_t)map[k];
    D.x[k] = S.x[m];
    D.y[k] = S.y[m];
    D.z[k] = S.z[m];
    D.ux[k] = S.ux[m];
    D.uy[k] = S.uy[m];
    D.uz[k] = S.uz[m];
    D.id[k] = S.id[m];
  }
}

void gather3d(const Dev3D& d, const Parts3D& src, const Parts3D& dst, const int* map, const int* counts,
              cudaStream_t s) {
  k_gather3d<<<d.nrow, 256, 0, s>>>(d, src, dst, map, counts);
}

// ---------------------------------------------------------------------------
// layout conversions between up(ndim, np, ny, nz, nsp) (AoS inside each row) and the device
// SoA; rows [row0, row0+nrows) of a staging block
// ---------------------------------------------------------------------------
__global__ void k_aos_to_soa3d(Dev3D d, const double* aos, int ndim, int np_host, int row0, Parts3D P) {
  const int row = row0 + blockIdx.x;  // one block per row of the staging block
  const int n = d.np2[row];
  for (int s = threadIdx.x; s < n; s += blockDim.x) {
    const double* a = aos + ((size_t)blockIdx.x * np_host + s) * ndim;
    const size_t k = (size_t)row * d.cap + s;
    P.x[k] = a[0];
    P.y[k] = a[1];
    P.z[k] = a[2];
    P.ux[k] = a[3];
    P.uy[k] = a[4];
    P.uz[k] = a[5];
    P.id[k] = ndim > 6 ? __double_as_longlong(a[6]) : 0;
  }
}

__global__ void k_soa_to_aos3d(Dev3D d, double* aos, int ndim, int np_host, int row0, Parts3D P) {
  const int row = row0 + blockIdx.x;
  const int n = d.np2[row];
  for (int s = threadIdx.x; s < n; s += blockDim.x) {
    double* a = aos + ((size_t)blockIdx.x * np_host + s) * ndim;
    const size_t k = (size_t)row * d.cap + s;
    a[0] = P.x[k];
    a[1] = P.y[k];
    a[2] = P.z[k];
    a[3] = P.ux[k];
    a[4] = P.uy[k];
    a[5] = P.uz[k];
    if (ndim > 6) a[6] = __longlong_as_double(P.id[k]);
  }
}

void aos_to_soa3d(const Dev3D& d, const double* aos, int ndim, int np_host, int row0, int nrows, const Parts3D& P,
                  cudaStream_t s) {
  k_aos_to_soa3d<<<nrows, 256, 0, s>>>(d, aos, ndim, np_host, row0, P);
}

void soa_to_aos3d(const Dev3D& d, double* aos, int ndim, int np_host, int row0, int nrows, const Parts3D& P,
                  cudaStream_t s) {
  k_soa_to_aos3d<<<nrows, 256, 0, s>>>(d, aos, ndim, np_host, row0, P);
}

// ---------------------------------------------------------------------------
// Device-side 3D Weibel loader: ppc particles per cell per species, uniform in the cell,
// cell-major inside each row (already bucket-sorted), co-located ion/electron pairs,
// electron beams +-drift alternating by particle; Philox4x32-10 counters (k, row, stream).
// ---------------------------------------------------------------------------
__global__ void k_load_weibel3d(Dev3D d, int ppc, unsigned long long seed, double drift, int axis, double u_thi,
                                double u_the) {
  const Grid3D g = d.g;
  const int rs = blockIdx.x;  // row within a species: kk * ny + jj (one block per row)
  const int jj = rs % g.ny, kk = rs / g.ny;
  const int npr = g.nx * ppc;
  const uint2 key = make_uint2((unsigned)seed, (unsigned)(seed >> 32));
  for (int k = threadIdx.x; k < npr || k <= g.nx; k += blockDim.x) {  // particle index in the row
  if (k < npr) {
    const int cx = k / ppc;
    const uint4 rp = philox4x32(make_uint4((unsigned)k, (unsigned)rs, 0u, 0u), key);
    const uint4 rz = philox4x32(make_uint4((unsigned)k, (unsigned)rs, 7u, 0u), key);
    // in-cell fractions on a 2^-40 grid in [0, 1): cell + fraction is exact, so int(x) is the cell
    auto frac = [](double u) { return floor((1.0 - u) * 1099511627776.0) * (1.0 / 1099511627776.0); };
    const double x = ((double)(g.nxgs + cx) + frac(u01(rp.x, rp.y))) * d.ph.delx;
    const double y = ((double)(g.nygs + jj) + frac(u01(rp.z, rp.w))) * d.ph.delx;
    const double z = ((double)(g.nzgs + kk) + frac(u01(rz.x, rz.y))) * d.ph.delx;
    for (int isp = 0; isp < d.ph.nsp; ++isp) {
      const int row = isp * g.ny * g.nz + rs;
      const size_t o = (size_t)row * d.cap + k;
      const uint4 r1 = philox4x32(make_uint4((unsigned)k, (unsigned)rs, 1u + 2u * isp, 0u), key);
      const uint4 r2 = philox4x32(make_uint4((unsigned)k, (unsigned)rs, 2u + 2u * isp, 0u), key);
      const double sd = isp == 0 ? u_thi : u_the;
      const double twopi = 6.283185307179586;
      const double a1 = u01(r1.x, r1.y), b1 = u01(r1.z, r1.w), a2 = u01(r2.x, r2.y), b2 = u01(r2.z, r2.w);
      const double rad1 = sqrt(-2.0 * log(a1)), rad2 = sqrt(-2.0 * log(a2));
      double u[3] = {sd * rad1 * cos(twopi * b1), sd * rad1 * sin(twopi * b1), sd * rad2 * cos(twopi * b2)};
      if (isp == 1 && drift != 0.0) u[axis] += (k % 2 == 0) ? drift : -drift;
      d.A.x[o] = x;
      d.A.y[o] = y;
      d.A.z[o] = z;
      d.A.ux[o] = u[0];
      d.A.uy[o] = u[1];
      d.A.uz[o] = u[2];
      d.A.id[o] = -((long long)rs * npr + k + 1);
    }
  }
  if (k <= g.nx)
    for (int isp = 0; isp < d.ph.nsp; ++isp) d.cc[(size_t)(isp * g.ny * g.nz + rs) * (g.nx + 1) + k] = k * ppc;
  if (k == 0)
    for (int isp = 0; isp < d.ph.nsp; ++isp) d.np2[isp * g.ny * g.nz + rs] = npr;
  }
}

void load_weibel3d_ppc(const Dev3D& d, int ppc, unsigned long long seed, double drift, int drift_axis,
                       double u_thi, double u_the, cudaStream_t s) {
  k_load_weibel3d<<<d.g.ny * d.g.nz, 256, 0, s>>>(d, ppc, seed, drift, drift_axis, u_thi, u_the);
}

// ---------------------------------------------------------------------------
// boundary_periodic__mom  (3d/common/boundary_periodic.f90:1102-1235), one rank:
// x images over every (j, k); the y self-exchange over every z layer; the z
// self-exchange over the interior y rows.  Three launches, in that order.
// ---------------------------------------------------------------------------
__global__ void k_mom3_fold_x(Dev3D d, double* mom) {
  const Grid3D g = d.g;
  const long long nxm = g.nx + 2;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;  // (l, jn, kn, isp)
  if (t >= 7LL * (g.ny + 2) * (g.nz + 2) * d.ph.nsp) return;
  const int l = (int)(t % 7);
  double* m = mom + (t / 7) * nxm * 7 + l;
  if (d.ph.bc == BC_PERIODIC) {
    m[7] = m[7] + m[7 * (size_t)(g.nx + 1)];
    m[7 * (size_t)g.nx] = m[7 * (size_t)g.nx] + m[0];
  } else {  // boundary_reconnection__mom (:1134-1137): the x ghosts onto the wall columns
    m[7] = m[7] + m[0];
    m[7 * (size_t)g.nx] = m[7 * (size_t)g.nx] + m[7 * (size_t)(g.nx + 1)];
  }
}

__global__ void k_mom3_fold_y(Dev3D d, double* mom) {
  const Grid3D g = d.g;
  const size_t rowst = 7 * (size_t)(g.nx + 2);               // stride of jn
  const size_t plane = rowst * (size_t)(g.ny + 2);           // stride of kn
  const int t = blockIdx.x * blockDim.x + threadIdx.x;       // (l, in)
  if (t >= (int)rowst) return;
  const int kn = blockIdx.y, isp = blockIdx.z;
  double* m = mom + ((size_t)isp * (g.nz + 2) + kn) * plane + t;
  m[rowst * g.ny] = m[rowst * g.ny] + m[0];
  m[rowst] = m[rowst] + m[rowst * (g.ny + 1)];
}

__global__ void k_mom3_fold_z(Dev3D d, double* mom) {
  const Grid3D g = d.g;
  const size_t rowst = 7 * (size_t)(g.nx + 2);
  const size_t plane = rowst * (size_t)(g.ny + 2);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;  // (l, in)
  if (t >= (int)rowst) return;
  const int jn = 1 + blockIdx.y, isp = blockIdx.z;      // interior rows nys..nye
  double* m = mom + (size_t)isp * (g.nz + 2) * plane + jn * rowst + t;
  m[plane * g.nz] = m[plane * g.nz] + m[0];
  m[plane] = m[plane] + m[plane * (g.nz + 1)];
}

void bc_mom3d(const Dev3D& d, double* mom, cudaStream_t s) {
  const long long nxt = 7LL * (d.g.ny + 2) * (d.g.nz + 2) * d.ph.nsp;
  const int rowst = 7 * (d.g.nx + 2);
  k_mom3_fold_x<<<(unsigned)((nxt + 255) / 256), 256, 0, s>>>(d, mom);
  k_mom3_fold_y<<<dim3((rowst + 255) / 256, d.g.nz + 2, d.ph.nsp), 256, 0, s>>>(d, mom);
  k_mom3_fold_z<<<dim3((rowst + 255) / 256, d.g.ny, d.ph.nsp), 256, 0, s>>>(d, mom);
}

}  // namespace wpic
