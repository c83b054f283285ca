// Discrete adjoint of the 2D FP64 time step (periodic boundaries), reverse mode, one step
// at a time.  The step is
//   push        B = P(A, uf)                       (2d/common/particle.f90:48-179)
//   deposit     J = D(A, B)                        (2d/common/field.f90:189-316)
//   fold        Jf = F(J)                          (boundary_periodic__curre)
//   field       uf' = uf + df,  df = E(uf, Jf)     (2d/common/field.f90:66-186: RHS, CG, E update)
//   bookkeeping A' = S(B)                          (particle_x, particle_y, sort: a permutation)
// and its adjoint, given the adjoints (lA', luf') of the state after the step, returns
// (lA, luf) of the state before it:
//   lB = S^T lA'                       (scatter through the permutation)
//   ldf = luf'; luf = luf'             (uf' = uf + df)
//   the field part backwards: ghost copies -> folds, E update -> its transposed stencil,
//   the CG -> one more CG solve with the same symmetric operator, RHS -> transposed stencil,
//   current fold -> its transpose: lJ
//   deposit: lA(x, y) and lB(x, y, u) += dJ/d(.)^T lJ
//   push:    lA += dB/dA^T lB, luf += dB/duf^T lB
// The push and the deposit are differentiated per particle in reverse mode, by hand, on the
// same expressions as the forward kernels (one backward sweep through the Boris rotation
// and through the Esirkepov weights gives all input adjoints at a few times the primal
// cost); the linear field operators are transposed by hand (the dot-product identity
// <L x, y> = <x, L^T y> is checked by wpic_adjoint_selfcheck).  The push's field adjoints
// are summed per cell inside each block and added to the nodes with FP64 atomics: the
// adjoint is reproducible to round-off, not bitwise.
#include <cmath>

#include "common.cuh"

namespace wpic {

namespace {

__device__ __forceinline__ int cell_of(const int* ccr, int nc, int s) {
  int lo = 0, hi = nc;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (ccr[mid] <= s) lo = mid; else hi = mid;
  }
  return lo;
}

}  // namespace

// cell-centred fields tmp(1:6, i, j) for cells -1..nx, -1..ny (2d/common/particle.f90:70-83)
__global__ void k_adj_tmp(Dev2D d, double* tmp) {
  const Grid2D g = d.g;
  const int tw = g.nx + 2, th = g.ny + 2;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < tw * th; t += gridDim.x * blockDim.x) {
    const int ci = t % tw, cj = t / tw;  // local cell (ci - 1, cj - 1): field index (ci + 1, cj + 1)
    const size_t b0 = (size_t)(cj + 1) * g.fp + (ci + 1), P = g.fplane;
    const double* U = d.uf;
    const size_t n = (size_t)tw * th;
    tmp[t] = 0.5 * (U[b0] + U[b0 + g.fp]);
    tmp[n + t] = 0.5 * (U[P + b0] + U[P + b0 + 1]);
    tmp[2 * n + t] = 0.25 * (U[2 * P + b0] + U[2 * P + b0 + 1] + U[2 * P + b0 + g.fp] + U[2 * P + b0 + g.fp + 1]);
    tmp[3 * n + t] = 0.5 * (U[3 * P + b0] + U[3 * P + b0 + 1]);
    tmp[4 * n + t] = 0.5 * (U[4 * P + b0] + U[4 * P + b0 + g.fp]);
    tmp[5 * n + t] = U[5 * P + b0];
  }
}

// luf += (the averaging of k_adj_tmp)^T ltmp
__global__ void k_adj_tmpT(Dev2D d, const double* ltmp, double* luf) {
  const Grid2D g = d.g;
  const int tw = g.nx + 2, th = g.ny + 2;
  const size_t n = (size_t)tw * th, P = g.fplane;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < tw * th; t += gridDim.x * blockDim.x) {
    const int ci = t % tw, cj = t / tw;
    const size_t b0 = (size_t)(cj + 1) * g.fp + (ci + 1);
    const double l0 = ltmp[t], l1 = ltmp[n + t], l2 = ltmp[2 * n + t];
    const double l3 = ltmp[3 * n + t], l4 = ltmp[4 * n + t], l5 = ltmp[5 * n + t];
    if (l0 != 0.0) { atomicAdd(luf + b0, 0.5 * l0); atomicAdd(luf + b0 + g.fp, 0.5 * l0); }
    if (l1 != 0.0) { atomicAdd(luf + P + b0, 0.5 * l1); atomicAdd(luf + P + b0 + 1, 0.5 * l1); }
    if (l2 != 0.0) {
      atomicAdd(luf + 2 * P + b0, 0.25 * l2);
      atomicAdd(luf + 2 * P + b0 + 1, 0.25 * l2);
      atomicAdd(luf + 2 * P + b0 + g.fp, 0.25 * l2);
      atomicAdd(luf + 2 * P + b0 + g.fp + 1, 0.25 * l2);
    }
    if (l3 != 0.0) { atomicAdd(luf + 3 * P + b0, 0.5 * l3); atomicAdd(luf + 3 * P + b0 + 1, 0.5 * l3); }
    if (l4 != 0.0) { atomicAdd(luf + 4 * P + b0, 0.5 * l4); atomicAdd(luf + 4 * P + b0 + g.fp, 0.5 * l4); }
    if (l5 != 0.0) atomicAdd(luf + 5 * P + b0, l5);
  }
}

// lB[map[k]] = lA'[k] over the valid slots of the sorted state after the step
__global__ void k_adj_unsort(Dev2D d, Parts64 lA, Parts64 lB, const int* map, const int* counts) {
  const int row = blockIdx.y;
  const int pos = blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= counts[row]) return;
  const size_t k = (size_t)row * d.cap + pos, m = (size_t)map[k];
  lB.x[m] = lA.x[k];
  lB.y[m] = lA.y[k];
  lB.ux[m] = lA.ux[k];
  lB.uy[m] = lA.uy[k];
  lB.uz[m] = lA.uz[k];
}

// ---- transposed ghost copies, folds and stencils (periodic) ----
// dfield_ghost2d copies interior rows/columns into the two ghost layers (y for interior
// columns, then x for every row); its transpose adds each ghost's adjoint into its source
// and clears it, x first.
__global__ void k_adj_dghost_x(Dev2D d, double* l, int ncomp) {
  const Grid2D g = d.g;
  const int jf = blockIdx.x * blockDim.x + threadIdx.x;
  if (jf >= g.ny + 4) return;
  const int nx = g.nx;
  for (int k = 0; k < ncomp; ++k) {
    double* u = l + (size_t)k * g.fplane + (size_t)jf * g.fp;
    u[nx] += u[0];
    u[0] = 0.0;
    u[nx + 1] += u[1];
    u[1] = 0.0;
    u[2] += u[nx + 2];
    u[nx + 2] = 0.0;
    u[3] += u[nx + 3];
    u[nx + 3] = 0.0;
  }
}
__global__ void k_adj_dghost_y(Dev2D d, double* l, int ncomp) {
  const Grid2D g = d.g;
  const int ii = 2 + blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= g.nx + 2) return;
  const int ny = g.ny;
  const size_t fp = g.fp;
  for (int k = 0; k < ncomp; ++k) {
    double* u = l + (size_t)k * g.fplane + ii;
    u[2 * fp] += u[(ny + 2) * fp];
    u[(ny + 2) * fp] = 0.0;
    u[3 * fp] += u[(ny + 3) * fp];
    u[(ny + 3) * fp] = 0.0;
    u[ny * fp] += u[0];
    u[0] = 0.0;
    u[(ny + 1) * fp] += u[fp];
    u[fp] = 0.0;
  }
}

// curre fold: interior t += ghost g, then ghost g := t (y for every column, then x for every
// row).  Transpose per pair: both become lt + lg; x first.
__global__ void k_adj_curre_x(Dev2D d, double* l) {
  const Grid2D g = d.g;
  const int jf = blockIdx.x * blockDim.x + threadIdx.x;
  if (jf >= g.ny + 4) return;
  const int nx = g.nx;
  for (int k = 0; k < 3; ++k) {
    double* u = l + (size_t)k * g.fplane + (size_t)jf * g.fp;
    const int tg[4][2] = {{nx, 0}, {nx + 1, 1}, {2, nx + 2}, {3, nx + 3}};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const double s = u[tg[q][0]] + u[tg[q][1]];
      u[tg[q][0]] = s;
      u[tg[q][1]] = s;
    }
  }
}
__global__ void k_adj_curre_y(Dev2D d, double* l) {
  const Grid2D g = d.g;
  const int ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= g.nx + 4) return;
  const int ny = g.ny;
  const size_t fp = g.fp;
  for (int k = 0; k < 3; ++k) {
    double* u = l + (size_t)k * g.fplane + ii;
    const size_t tg[4][2] = {{ny * fp, 0}, {(ny + 1) * fp, fp}, {2 * fp, (ny + 2) * fp}, {3 * fp, (ny + 3) * fp}};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const double s = u[tg[q][0]] + u[tg[q][1]];
      u[tg[q][0]] = s;
      u[tg[q][1]] = s;
    }
  }
}

// E update (2d/common/field.f90:153-171) transposed: ldf(3..5) at the cell -> ldf(0..2)
// (ghosts included), luf, luj; ldf(3..5) at the cell consumed
__global__ void k_adj_efield(Dev2D d, double* ldf, double* luf, double* luj) {
  const Grid2D g = d.g;
  const int cx = blockIdx.x * blockDim.x + threadIdx.x, cy = blockIdx.y;
  if (cx >= g.nx) return;
  const size_t f = (size_t)(cy + 2) * g.fp + (cx + 2), P = g.fplane;
  const size_t E = f + 1, N = f + g.fp;
  const double f1 = d.ph.f1, gf = d.ph.gfac, fj = 4. * d.ph.pi * d.ph.delt;
  const double l4 = ldf[3 * P + f], l5 = ldf[4 * P + f], l6 = ldf[5 * P + f];
  ldf[3 * P + f] = 0.0;
  ldf[4 * P + f] = 0.0;
  ldf[5 * P + f] = 0.0;
  // d4 = f1 (gf (-D2(f) + D2(N)) + (-U2(f) + U2(N))) - fj J0(f)
  atomicAdd(ldf + 2 * P + f, -f1 * gf * l4 + f1 * gf * l5);
  atomicAdd(ldf + 2 * P + N, f1 * gf * l4);
  atomicAdd(luf + 2 * P + f, -f1 * l4 + f1 * l5);
  atomicAdd(luf + 2 * P + N, f1 * l4);
  atomicAdd(luj + f, -fj * l4);
  // d5 = -f1 (gf (-D2(f) + D2(E)) + (-U2(f) + U2(E))) - fj J1(f)
  atomicAdd(ldf + 2 * P + E, -f1 * gf * l5);
  atomicAdd(luf + 2 * P + E, -f1 * l5);
  atomicAdd(luj + P + f, -fj * l5);
  // d6 = f1 (gf (-D1(f) + D1(E) + D0(f) - D0(N)) + (-U1(f) + U1(E) + U0(f) - U0(N))) - fj J2(f)
  atomicAdd(ldf + P + f, -f1 * gf * l6);
  atomicAdd(ldf + P + E, f1 * gf * l6);
  atomicAdd(ldf + f, f1 * gf * l6);
  atomicAdd(ldf + N, -f1 * gf * l6);
  atomicAdd(luf + P + f, -f1 * l6);
  atomicAdd(luf + P + E, f1 * l6);
  atomicAdd(luf + f, f1 * l6);
  atomicAdd(luf + N, -f1 * l6);
  atomicAdd(luj + 2 * P + f, -fj * l6);
}

// RHS gkl (2d/common/field.f90:125-146) transposed: lgkl -> luf, luj
__global__ void k_adj_gkl(Dev2D d, const double* lg, double* luf, double* luj) {
  const Grid2D g = d.g;
  const int cx = blockIdx.x * blockDim.x + threadIdx.x, cy = blockIdx.y;
  if (cx >= g.nx) return;
  const size_t f = (size_t)(cy + 2) * g.fp + (cx + 2), P = g.fplane;
  const size_t S = f - g.fp, W = f - 1, E = f + 1, N = f + g.fp;
  const double f1 = d.ph.f1, f2 = d.ph.f2, f3 = d.ph.f3;
  const size_t c = (size_t)cy * g.nx + cx;
  const double l1 = lg[c], l2 = lg[(size_t)g.ncell + c], l3 = lg[2 * (size_t)g.ncell + c];
  // g1 = f2 (U0(S)+U0(W)-4U0(f)+U0(E)+U0(N) + f3 (-J2(S)+J2(f))) - f1 (-U5(S)+U5(f))
  atomicAdd(luf + S, f2 * l1);
  atomicAdd(luf + W, f2 * l1);
  atomicAdd(luf + f, -4. * f2 * l1);
  atomicAdd(luf + E, f2 * l1);
  atomicAdd(luf + N, f2 * l1);
  atomicAdd(luj + 2 * P + S, -f2 * f3 * l1);
  atomicAdd(luj + 2 * P + f, f2 * f3 * l1);
  atomicAdd(luf + 5 * P + S, f1 * l1);
  atomicAdd(luf + 5 * P + f, -f1 * l1);
  // g2 = f2 (U1(S)+U1(W)-4U1(f)+U1(E)+U1(N) - f3 (-J2(W)+J2(f))) + f1 (-U5(W)+U5(f))
  atomicAdd(luf + P + S, f2 * l2);
  atomicAdd(luf + P + W, f2 * l2);
  atomicAdd(luf + P + f, -4. * f2 * l2);
  atomicAdd(luf + P + E, f2 * l2);
  atomicAdd(luf + P + N, f2 * l2);
  atomicAdd(luj + 2 * P + W, f2 * f3 * l2);
  atomicAdd(luj + 2 * P + f, -f2 * f3 * l2);
  atomicAdd(luf + 5 * P + W, -f1 * l2);
  atomicAdd(luf + 5 * P + f, f1 * l2);
  // g3 = f2 (U2(S)+U2(W)-4U2(f)+U2(E)+U2(N) + f3 (-J1(W)+J1(f)+J0(S)-J0(f))) - f1 (-U4(W)+U4(f)+U3(S)-U3(f))
  atomicAdd(luf + 2 * P + S, f2 * l3);
  atomicAdd(luf + 2 * P + W, f2 * l3);
  atomicAdd(luf + 2 * P + f, -4. * f2 * l3);
  atomicAdd(luf + 2 * P + E, f2 * l3);
  atomicAdd(luf + 2 * P + N, f2 * l3);
  atomicAdd(luj + P + W, -f2 * f3 * l3);
  atomicAdd(luj + P + f, f2 * f3 * l3);
  atomicAdd(luj + S, f2 * f3 * l3);
  atomicAdd(luj + f, -f2 * f3 * l3);
  atomicAdd(luf + 4 * P + W, f1 * l3);
  atomicAdd(luf + 4 * P + f, -f1 * l3);
  atomicAdd(luf + 3 * P + S, -f1 * l3);
  atomicAdd(luf + 3 * P + f, f1 * l3);
}

// the CG solution of the adjoint solve is the RHS of k_cg_init (b = f5 gkl): set gkl = ldb
// (interior of ldf(0..2)) and the warm start to zero
__global__ void k_adj_cg_setup(Dev2D d, const double* ldf) {
  const Grid2D g = d.g;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < g.ncell; c += gridDim.x * blockDim.x) {
    const int cy = c / g.nx, cx = c - cy * g.nx;
    const size_t f = (size_t)(cy + 2) * g.fp + cx + 2;
    for (int l = 0; l < 3; ++l) {
      d.gkl[(size_t)l * g.ncell + c] = ldf[(size_t)l * g.fplane + f];
      d.df[(size_t)l * g.fplane + f] = 0.0;
    }
  }
}
__global__ void k_adj_cg_result(Dev2D d, double* lg) {
  const Grid2D g = d.g;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < g.ncell; c += gridDim.x * blockDim.x) {
    const int cy = c / g.nx, cx = c - cy * g.nx;
    for (int l = 0; l < 3; ++l)
      lg[(size_t)l * g.ncell + c] = d.df[(size_t)l * g.fplane + (size_t)(cy + 2) * g.fp + cx + 2];
  }
}

// reciprocal square root in the kernel's arithmetic type
__device__ __forceinline__ double rsq(double v) { return rsqrt(v); }
__device__ __forceinline__ float rsq(float v) { return rsqrtf(v); }

// ---- the deposit's adjoint: inputs (x_old, y_old, x_new, y_new, ux', uy', uz') ----
// Forward (per particle, 2d/common/field.f90:189-316): shapes s0 (old position, 5-point
// stencil around the old cell), S1 (new position, shifted by the cell change inc), ds = S1 - s0,
//   Jx(i+1, j) = -qdd wy[j] sum_{i'<=i} ds_x[i'],   wy = s0_y + ds_y / 2,
//   Jy(i, j+1) = -qdd wx[i] sum_{j'<=j} ds_y[j'],   wx = s0_x + ds_x / 2,
//   Jz(i, j)   = q gvz (s0_x s0_y + ds_x s0_y / 2 + s0_x ds_y / 2 + ds_x ds_y / 3),
// gvz = uz / sqrt(1 + u^2 / c^2).  Reverse: the adjoints of the 5-point shape arrays from
// suffix sums of lJ, then through ds = S1 - s0, the shift and the quadratic spline.
// R is the arithmetic type of the per-particle sweep: double, or float for the
// mixed-precision adjoint (lJ then comes as an FP32 copy, made once per step, so that no
// particle converts field values).  The in-cell offsets and the cell indices come from the
// FP64 positions in FP64 either way; the particle adjoints are accumulated into FP64 arrays.
template <typename R>
__global__ void __launch_bounds__(128) k_adj_deposit(Dev2D d, const R* luj, Parts64 lA, Parts64 lB) {
  const Grid2D g = d.g;
  const int row = blockIdx.y;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= d.np2[row]) return;
  const int isp = row / g.ny, jj = row - isp * g.ny;
  const int* ccr = d.cc + (size_t)row * (g.nx + 1);
  const int cx = cell_of(ccr, g.nx, s);
  const size_t k = (size_t)row * d.cap + s;
  const double d_delx = d.ph.d_delx;
  const R dxr = (R)d_delx, c = (R)d.ph.c, q = (R)d.ph.q[isp];
  const R qdd = (R)(d.ph.q[isp] * d.ph.delx * d.ph.d_delt), fac = R(1) / R(3);
  const R h5 = R(0.5), q34 = R(0.75);
  const int iabs = g.nxgs + cx, jabs = g.nygs + jj;
  const double pos0[2] = {d.A.x[k], d.A.y[k]};
  const double pos1[2] = {d.B.x[k], d.B.y[k]};
  R s0[2][5], ds[2][5], dh[2], dh1[2];
  int inc[2];
#pragma unroll
  for (int dim = 0; dim < 2; ++dim) {
    const R h = (R)(d_delx * pos0[dim] + (-0.5 - (double)(dim == 0 ? iabs : jabs)));
    dh[dim] = h;
    s0[dim][0] = R(0);
    s0[dim][1] = h5 * ((h5 - h) * (h5 - h));
    s0[dim][2] = q34 - h * h;
    s0[dim][3] = h5 * ((h5 + h) * (h5 + h));
    s0[dim][4] = R(0);
    const int i2 = (int)(pos1[dim] * d_delx);
    const R h1 = (R)(d_delx * pos1[dim] + (-0.5 - (double)i2));
    dh1[dim] = h1;
    inc[dim] = i2 - (dim == 0 ? iabs : jabs);
    const R a1 = h5 * ((h5 - h1) * (h5 - h1)), a2 = q34 - h1 * h1, a3 = h5 * ((h5 + h1) * (h5 + h1));
    const int ai = inc[dim] < 0 ? -inc[dim] : inc[dim];
    const R m1 = (R)(-(inc[dim] - ai)) * h5, m2 = (R)(-ai + 1), m3 = (R)(inc[dim] + ai) * h5;
    ds[dim][0] = m1 * a1 - s0[dim][0];
    ds[dim][1] = m2 * a1 + m1 * a2 - s0[dim][1];
    ds[dim][2] = m2 * a2 + m1 * a3 + m3 * a1 - s0[dim][2];
    ds[dim][3] = m2 * a3 + m3 * a2 - s0[dim][3];
    ds[dim][4] = m3 * a3 - s0[dim][4];
  }
  const R ux = (R)d.B.ux[k], uy = (R)d.B.uy[k], uz = (R)d.B.uz[k];
  const R ic2 = R(1) / (c * c);
  const R gmi = rsq(R(1) + ic2 * (ux * ux + uy * uy + uz * uz));
  const R gvz = uz * gmi;
  const size_t P = g.fplane;
  const R* L0 = luj + (size_t)jj * g.fp + cx;  // node (cx + a, jj + b) at L0[b * fp + a]
  R gs0[2][5], gds[2][5];
#pragma unroll
  for (int dim = 0; dim < 2; ++dim)
#pragma unroll
    for (int i = 0; i < 5; ++i) gs0[dim][i] = gds[dim][i] = R(0);
  // Jx: nodes (i + 1, j), i = 0..3, j = 0..4.  With Px the prefix sums of ds_x and
  // Rx_i = sum_j wy_j lJx(i + 1, j): the adjoint of ds_x(i') is -qdd sum_{i >= i'} Rx_i, that of
  // wy_j is -qdd sum_i Px_i lJx(i + 1, j) -- each lJx entry read once into two fused
  // multiply-adds
  const R wy[5] = {s0[1][0] + h5 * ds[1][0], s0[1][1] + h5 * ds[1][1], s0[1][2] + h5 * ds[1][2],
                   s0[1][3] + h5 * ds[1][3], s0[1][4] + h5 * ds[1][4]};
  const R wx[5] = {s0[0][0] + h5 * ds[0][0], s0[0][1] + h5 * ds[0][1], s0[0][2] + h5 * ds[0][2],
                   s0[0][3] + h5 * ds[0][3], s0[0][4] + h5 * ds[0][4]};
  {
    R Px[4], Rx[4], gwy[5] = {R(0), R(0), R(0), R(0), R(0)};
    Px[0] = ds[0][0];
#pragma unroll
    for (int q = 1; q < 4; ++q) Px[q] = Px[q - 1] + ds[0][q];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      R r = R(0);
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        const R l = L0[(size_t)j * g.fp + i + 1];
        r += wy[j] * l;
        gwy[j] += Px[i] * l;
      }
      Rx[i] = r;
    }
    R suf = R(0);
#pragma unroll
    for (int i = 3; i >= 0; --i) {
      suf += Rx[i];
      gds[0][i] += -qdd * suf;
    }
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      const R gw = -qdd * gwy[j];
      gs0[1][j] += gw;
      gds[1][j] += h5 * gw;
    }
  }
  // Jy: nodes (i, j + 1), i = 0..4, j = 0..3, the same with the axes exchanged
  const R* L1 = L0 + P;
  {
    R Py[4], Ry[4], gwx[5] = {R(0), R(0), R(0), R(0), R(0)};
    Py[0] = ds[1][0];
#pragma unroll
    for (int q = 1; q < 4; ++q) Py[q] = Py[q - 1] + ds[1][q];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      R r = R(0);
#pragma unroll
      for (int i = 0; i < 5; ++i) {
        const R l = L1[(size_t)(j + 1) * g.fp + i];
        r += wx[i] * l;
        gwx[i] += Py[j] * l;
      }
      Ry[j] = r;
    }
    R suf = R(0);
#pragma unroll
    for (int j = 3; j >= 0; --j) {
      suf += Ry[j];
      gds[1][j] += -qdd * suf;
    }
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      const R gw = -qdd * gwx[i];
      gs0[0][i] += gw;
      gds[0][i] += h5 * gw;
    }
  }
  // Jz: nodes (i, j) = Qz (s0_x (x) Ay + ds_x (x) By), Ay = s0_y + ds_y / 2, By = s0_y / 2 + ds_y / 3
  const R* L2 = L0 + 2 * P;
  const R Qz = q * gvz;
  R gAy[5] = {R(0), R(0), R(0), R(0), R(0)}, gBy[5] = {R(0), R(0), R(0), R(0), R(0)}, phiz = R(0);
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    R r1 = R(0), r2 = R(0);
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      const R l = L2[(size_t)j * g.fp + i];
      r1 += l * (s0[1][j] + h5 * ds[1][j]);
      r2 += l * (h5 * s0[1][j] + fac * ds[1][j]);
      if (i != 0 && i != 4) gAy[j] += l * s0[0][i];  // s0 is zero at the stencil's ends
      gBy[j] += l * ds[0][i];
    }
    gs0[0][i] += Qz * r1;
    gds[0][i] += Qz * r2;
    phiz += s0[0][i] * r1 + ds[0][i] * r2;
  }
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    gs0[1][j] += Qz * (gAy[j] + h5 * gBy[j]);
    gds[1][j] += Qz * (h5 * gAy[j] + fac * gBy[j]);
  }
  // through ds = S1 - s0, the shift by inc and the splines
  R gpos0[2], gpos1[2];
#pragma unroll
  for (int dim = 0; dim < 2; ++dim) {
    const int ai = inc[dim] < 0 ? -inc[dim] : inc[dim];
    const R m1 = (R)(-(inc[dim] - ai)) * h5, m2 = (R)(-ai + 1), m3 = (R)(inc[dim] + ai) * h5;
    const R ga1 = m1 * gds[dim][0] + m2 * gds[dim][1] + m3 * gds[dim][2];
    const R ga2 = m1 * gds[dim][1] + m2 * gds[dim][2] + m3 * gds[dim][3];
    const R ga3 = m1 * gds[dim][2] + m2 * gds[dim][3] + m3 * gds[dim][4];
    const R h1 = dh1[dim], h = dh[dim];
    gpos1[dim] = dxr * (-(h5 - h1) * ga1 - R(2) * h1 * ga2 + (h5 + h1) * ga3);
    const R g1 = gs0[dim][1] - gds[dim][1], g2 = gs0[dim][2] - gds[dim][2], g3 = gs0[dim][3] - gds[dim][3];
    gpos0[dim] = dxr * (-(h5 - h) * g1 - R(2) * h * g2 + (h5 + h) * g3);
  }
  // gvz = uz / gamma
  const R ggv = q * phiz;
  const R t3 = gmi * gmi * gmi * ic2 * uz;
  lA.x[k] += (double)gpos0[0];
  lA.y[k] += (double)gpos0[1];
  lB.x[k] += (double)gpos1[0];
  lB.y[k] += (double)gpos1[1];
  lB.ux[k] += (double)(ggv * (-t3 * ux));
  lB.uy[k] += (double)(ggv * (-t3 * uy));
  lB.uz[k] += (double)(ggv * (gmi - t3 * uz));
}

// ---- the push's adjoint: inputs (x, y, ux, uy, uz) and the cell-centred fields tmp ----
// Forward (2d/common/particle.f90:48-179): gather B, E at the old position (quadratic
// splines on the cell-centred tmp), u1 = u + f1 E, gam = sqrt(c^2 + u1^2),
// w = u1 + (f1 / gam) u1 x B, u2 = u1 + f2 / (gam + f1^2 B^2 / gam) w x B, u' = u2 + f1 E,
// x' = x + dt u'_x / gamma', y' = y + dt u'_y / gamma'.  Reverse sweep through these lines;
// the field adjoints (B, E at the particle) spread back over the 3 x 3 tmp nodes with the
// same spline weights: summed per (cell, component, node) over the block's particles in
// shared memory (in R), then one FP64 atomic per (cell, component, node) of the block.
// For R = float the cell-centred fields come as an FP32 copy made once per step.
constexpr int AP_T = 128;
template <typename R>
__global__ void __launch_bounds__(AP_T) k_adj_push(Dev2D d, const R* tmp, Parts64 lA, Parts64 lB,
                                                   double* ltmp) {
  // per particle of the block: lf_m sy_b (the field adjoint times the y weight of node row b)
  // and sx_a, so that each (cell, component, node) sum takes one fused multiply-add per particle
  __shared__ R sq[18][AP_T + 1];
  __shared__ R sxs[3][AP_T + 1];
  const Grid2D g = d.g;
  const int row = blockIdx.y;
  const int s0b = blockIdx.x * AP_T;
  const int np = d.np2[row];
  if (s0b >= np) return;  // uniform across the block
  const int tid = threadIdx.x;
  const int s = s0b + tid;
  const int isp = row / g.ny, jj = row - isp * g.ny;
  const int* ccr = d.cc + (size_t)row * (g.nx + 1);
  const int tw = g.nx + 2;
  const size_t n = (size_t)tw * (g.ny + 2);
  if (s < np) {
    const int cx = cell_of(ccr, g.nx, s);
    const size_t k = (size_t)row * d.cap + s;
    const double dxi64 = d.ph.p_d_delx;
    const R dxi = (R)dxi64, delt = (R)d.ph.delt, c = (R)d.ph.c;
    const R fac1 = (R)(d.ph.q[isp] / d.ph.r[isp] * 0.5 * d.ph.delt);
    const R txxx = fac1 * fac1;
    const R fac2 = (R)(d.ph.q[isp] * d.ph.delt / d.ph.r[isp]);
    const R h5 = R(0.5), q34 = R(0.75), two = R(2);
    const int iabs = g.nxgs + cx, jabs = g.nygs + jj;
    const R hx = (R)(d.A.x[k] * dxi64 - 0.5 - (double)iabs), hy = (R)(d.A.y[k] * dxi64 - 0.5 - (double)jabs);
    const R sx[3] = {h5 * (h5 - hx) * (h5 - hx), q34 - hx * hx, h5 * (h5 + hx) * (h5 + hx)};
    const R sy[3] = {h5 * (h5 - hy) * (h5 - hy), q34 - hy * hy, h5 * (h5 + hy) * (h5 + hy)};
    const R dsx[3] = {-(h5 - hx) * dxi, -two * hx * dxi, (h5 + hx) * dxi};
    const R dsy[3] = {-(h5 - hy) * dxi, -two * hy * dxi, (h5 + hy) * dxi};
    // tmp node (a, b) of the particle's cell: local cell (cx - 1 + a, jj - 1 + b) -> index (cx + a, jj + b)
    R fv[6], fdx[6], fdy[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      R v = R(0), vx = R(0), vy = R(0);
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        R r = R(0), rx = R(0);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const R t = tmp[(size_t)m * n + (size_t)(jj + b) * tw + (cx + a)];
          r += t * sx[a];
          rx += t * dsx[a];
        }
        v += r * sy[b];
        vx += rx * sy[b];
        vy += r * dsy[b];
      }
      fv[m] = v;
      fdx[m] = vx;
      fdy[m] = vy;
    }
    const R B[3] = {fv[0], fv[1], fv[2]};
    const R ux = (R)d.A.ux[k], uy = (R)d.A.uy[k], uz = (R)d.A.uz[k];
    // forward values
    const R u1[3] = {ux + fac1 * fv[3], uy + fac1 * fv[4], uz + fac1 * fv[5]};
    const R gsq = c * c + (u1[0] * u1[0] + u1[1] * u1[1] + u1[2] * u1[2]);
    const R igam = rsq(gsq);
    const R gam = gsq * igam;
    const R fac1r = fac1 * igam;
    const R Bsq = B[0] * B[0] + B[1] * B[1] + B[2] * B[2];
    const R D = gam + txxx * (Bsq * igam);
    const R iD = R(1) / D;
    const R fac2r = fac2 * iD;
    const R u1xB[3] = {u1[1] * B[2] - u1[2] * B[1], u1[2] * B[0] - u1[0] * B[2], u1[0] * B[1] - u1[1] * B[0]};
    const R w[3] = {u1[0] + fac1r * u1xB[0], u1[1] + fac1r * u1xB[1], u1[2] + fac1r * u1xB[2]};
    const R wxB[3] = {w[1] * B[2] - w[2] * B[1], w[2] * B[0] - w[0] * B[2], w[0] * B[1] - w[1] * B[0]};
    const R gv[3] = {u1[0] + fac2r * wxB[0] + fac1 * fv[3], u1[1] + fac2r * wxB[1] + fac1 * fv[4],
                     u1[2] + fac2r * wxB[2] + fac1 * fv[5]};
    const R ic2 = R(1) / (c * c);
    const R gi = rsq(R(1) + ic2 * (gv[0] * gv[0] + gv[1] * gv[1] + gv[2] * gv[2]));
    // reverse
    const R lx = (R)lB.x[k], ly = (R)lB.y[k];
    const R gib = delt * (lx * gv[0] + ly * gv[1]);
    const R kk = gi * gi * gi * gib * ic2;
    R gb[3] = {(R)lB.ux[k] + delt * gi * lx - kk * gv[0], (R)lB.uy[k] + delt * gi * ly - kk * gv[1],
               (R)lB.uz[k] - kk * gv[2]};  // adjoint of u' (= of u2)
    R Eb[3] = {fac1 * gb[0], fac1 * gb[1], fac1 * gb[2]};
    const R f2rb = gb[0] * wxB[0] + gb[1] * wxB[1] + gb[2] * wxB[2];
    const R wb[3] = {fac2r * (B[1] * gb[2] - B[2] * gb[1]), fac2r * (B[2] * gb[0] - B[0] * gb[2]),
                     fac2r * (B[0] * gb[1] - B[1] * gb[0])};
    R Bb[3] = {fac2r * (gb[1] * w[2] - gb[2] * w[1]), fac2r * (gb[2] * w[0] - gb[0] * w[2]),
               fac2r * (gb[0] * w[1] - gb[1] * w[0])};
    R u1b[3] = {gb[0] + wb[0] + fac1r * (B[1] * wb[2] - B[2] * wb[1]),
                gb[1] + wb[1] + fac1r * (B[2] * wb[0] - B[0] * wb[2]),
                gb[2] + wb[2] + fac1r * (B[0] * wb[1] - B[1] * wb[0])};
    Bb[0] += fac1r * (wb[1] * u1[2] - wb[2] * u1[1]);
    Bb[1] += fac1r * (wb[2] * u1[0] - wb[0] * u1[2]);
    Bb[2] += fac1r * (wb[0] * u1[1] - wb[1] * u1[0]);
    const R f1rb = wb[0] * u1xB[0] + wb[1] * u1xB[1] + wb[2] * u1xB[2];
    const R Db = -(fac2r * iD) * f2rb;
    const R bsqb = Db * txxx * igam;
    Bb[0] += two * bsqb * B[0];
    Bb[1] += two * bsqb * B[1];
    Bb[2] += two * bsqb * B[2];
    const R igb = Db * txxx * Bsq + fac1 * f1rb;
    const R gamb = Db - igam * igam * igb;
    u1b[0] += gamb * igam * u1[0];
    u1b[1] += gamb * igam * u1[1];
    u1b[2] += gamb * igam * u1[2];
    Eb[0] += fac1 * u1b[0];
    Eb[1] += fac1 * u1b[1];
    Eb[2] += fac1 * u1b[2];
    const R lf[6] = {Bb[0], Bb[1], Bb[2], Eb[0], Eb[1], Eb[2]};
    R lxa = R(0), lya = R(0);
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      lxa += lf[m] * fdx[m];
      lya += lf[m] * fdy[m];
#pragma unroll
      for (int b = 0; b < 3; ++b) sq[m * 3 + b][tid] = lf[m] * sy[b];
    }
    // lA(x, y) = lB(x, y) + the gather's position derivative; the pass-through part in FP64
    lA.x[k] += lB.x[k] + (double)lxa;
    lA.y[k] += lB.y[k] + (double)lya;
    lA.ux[k] += (double)u1b[0];
    lA.uy[k] += (double)u1b[1];
    lA.uz[k] += (double)u1b[2];
#pragma unroll
    for (int a = 0; a < 3; ++a) sxs[a][tid] = sx[a];
  }
  __syncthreads();
  // per (cell, component, node) sums over the block's particles of each cell
  const int last = min(s0b + AP_T, np) - 1;
  const int c_first = cell_of(ccr, g.nx, s0b), c_last = cell_of(ccr, g.nx, last);
  const int nent = (c_last - c_first + 1) * 54;
  for (int e = tid; e < nent; e += AP_T) {
    const int cc = c_first + e / 54, r = e - (e / 54) * 54;
    const int m = r / 9, ab = r - m * 9, b = ab / 3, a = ab - b * 3;
    const int p0 = max(ccr[cc], s0b) - s0b, p1 = min(ccr[cc + 1], last + 1) - s0b;
    R acc = R(0);
    for (int p = p0; p < p1; ++p) acc += sq[m * 3 + b][p] * sxs[a][p];
    if (acc != R(0)) atomicAdd(ltmp + (size_t)m * n + (size_t)(jj + b) * tw + (cc + a), (double)acc);
  }
}

// ---- host-side sequences ----
void adj_field(const Dev2D& d, double* luf, double* ldf, double* luj, cudaStream_t s) {
  const Grid2D& g = d.g;
  const size_t P = g.fplane;
  cudaMemcpyAsync(ldf, luf, sizeof(double) * 6 * P, cudaMemcpyDeviceToDevice, s);  // uf' = uf + df
  cudaMemsetAsync(luj, 0, sizeof(double) * 3 * P, s);
  k_adj_dghost_x<<<(g.ny + 4 + 127) / 128, 128, 0, s>>>(d, ldf, 6);
  k_adj_dghost_y<<<(g.nx + 127) / 128, 128, 0, s>>>(d, ldf, 6);
  k_adj_efield<<<dim3((g.nx + 127) / 128, g.ny), 128, 0, s>>>(d, ldf, luf, luj);
  k_adj_dghost_x<<<(g.ny + 4 + 127) / 128, 128, 0, s>>>(d, ldf, 6);
  k_adj_dghost_y<<<(g.nx + 127) / 128, 128, 0, s>>>(d, ldf, 6);
  k_adj_cg_setup<<<4 * 152, 256, 0, s>>>(d, ldf);
}

void adj_field_after_cg(const Dev2D& d, double* luf, double* lg, double* luj, cudaStream_t s) {
  const Grid2D& g = d.g;
  k_adj_cg_result<<<4 * 152, 256, 0, s>>>(d, lg);
  k_adj_gkl<<<dim3((g.nx + 127) / 128, g.ny), 128, 0, s>>>(d, lg, luf, luj);
  k_adj_curre_x<<<(g.ny + 4 + 127) / 128, 128, 0, s>>>(d, luj);
  k_adj_curre_y<<<(g.nx + 4 + 127) / 128, 128, 0, s>>>(d, luj);
}

// the pieces on their own, for the dot-product checks
void adj_field_fold_T(const Dev2D& d, double* luj, cudaStream_t s) {
  k_adj_curre_x<<<(d.g.ny + 4 + 127) / 128, 128, 0, s>>>(d, luj);
  k_adj_curre_y<<<(d.g.nx + 4 + 127) / 128, 128, 0, s>>>(d, luj);
}
void adj_field_ghost_T(const Dev2D& d, double* ldf, cudaStream_t s) {
  k_adj_dghost_x<<<(d.g.ny + 4 + 127) / 128, 128, 0, s>>>(d, ldf, 6);
  k_adj_dghost_y<<<(d.g.nx + 127) / 128, 128, 0, s>>>(d, ldf, 6);
}
void adj_field_efield_T(const Dev2D& d, double* ldf, double* luf, double* luj, cudaStream_t s) {
  k_adj_efield<<<dim3((d.g.nx + 127) / 128, d.g.ny), 128, 0, s>>>(d, ldf, luf, luj);
}
void adj_field_gkl_T(const Dev2D& d, const double* lg, double* luf, double* luj, cudaStream_t s) {
  k_adj_gkl<<<dim3((d.g.nx + 127) / 128, d.g.ny), 128, 0, s>>>(d, lg, luf, luj);
}
void adj_field_tmp(const Dev2D& d, double* tmp, cudaStream_t s) { k_adj_tmp<<<4 * 152, 256, 0, s>>>(d, tmp); }
void adj_field_tmp_T(const Dev2D& d, const double* ltmp, double* luf, cudaStream_t s) {
  k_adj_tmpT<<<4 * 152, 256, 0, s>>>(d, ltmp, luf);
}

namespace {
__global__ void k_axpy(double* dst, const double* x, const double* v, double h, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = x[i] + h * v[i];
}
__global__ void k_dot_parts(Dev2D d, Parts64 L, Parts64 P, double scale, double* out) {
  const int row = blockIdx.y;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (s < d.np2[row]) {
    const size_t k = (size_t)row * d.cap + s;
    v = L.x[k] * P.x[k] + L.y[k] * P.y[k] + L.ux[k] * P.ux[k] + L.uy[k] * P.uy[k] + L.uz[k] * P.uz[k];
  }
  atomicAdd(out, scale * v);
}
}  // namespace

void adj_axpy(double* dst, const double* x, const double* v, double h, size_t n, cudaStream_t s) {
  k_axpy<<<4 * 152, 256, 0, s>>>(dst, x, v, h, n);
}
void adj_dot_parts(const Dev2D& d, const Parts64& L, const Parts64& P, double scale, double* out, cudaStream_t s) {
  k_dot_parts<<<dim3((d.cap + 255) / 256, d.nrowjob), 256, 0, s>>>(d, L, P, scale, out);
}
// FP32 copy of a field array for the FP32 sweeps
__global__ void k_to_f32(const double* a, float* b, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

namespace {
// the push's adjoint on the cell-centred fields tmp; f32 (null: FP64 sweep) holds 6 tmp planes
void launch_adj_push(const Dev2D& d, double* tmp, const Parts64& lA, const Parts64& lB, double* ltmp, float* f32,
                     cudaStream_t s) {
  const size_t n = (size_t)(d.g.nx + 2) * (d.g.ny + 2);
  dim3 grid((d.cap + 127) / 128, d.nrowjob);
  if (f32) {
    k_to_f32<<<4 * 152, 256, 0, s>>>(tmp, f32, 6 * n);
    k_adj_push<float><<<grid, 128, 0, s>>>(d, f32, lA, lB, ltmp);
  } else {
    k_adj_push<double><<<grid, 128, 0, s>>>(d, tmp, lA, lB, ltmp);
  }
}
void launch_adj_deposit(const Dev2D& d, const double* luj, const Parts64& lA, const Parts64& lB, float* f32,
                        cudaStream_t s) {
  dim3 grid((d.cap + 127) / 128, d.nrowjob);
  if (f32) {
    k_to_f32<<<4 * 152, 256, 0, s>>>(luj, f32, 3 * d.g.fplane);
    k_adj_deposit<float><<<grid, 128, 0, s>>>(d, f32, lA, lB);
  } else {
    k_adj_deposit<double><<<grid, 128, 0, s>>>(d, luj, lA, lB);
  }
}
}  // namespace

// the push's field adjoint alone: luf += (dB/duf)^T lB (lA receives the particle part)
void adj_push_fields(const Dev2D& d, const Parts64& lB, const Parts64& lA, double* tmp, double* ltmp, double* luf,
                     float* f32, cudaStream_t s) {
  const size_t n = (size_t)(d.g.nx + 2) * (d.g.ny + 2);
  k_adj_tmp<<<4 * 152, 256, 0, s>>>(d, tmp);
  cudaMemsetAsync(ltmp, 0, sizeof(double) * 6 * n, s);
  launch_adj_push(d, tmp, lA, lB, ltmp, f32, s);
  k_adj_tmpT<<<4 * 152, 256, 0, s>>>(d, ltmp, luf);
}

void adj_deposit_only(const Dev2D& d, const double* luj, const Parts64& lA, const Parts64& lB, float* f32,
                      cudaStream_t s) {
  launch_adj_deposit(d, luj, lA, lB, f32, s);
}

// zero everything but the interior cells of ncomp field planes
__global__ void k_keep_interior(Dev2D d, double* v, int ncomp) {
  const Grid2D g = d.g;
  const size_t n = (size_t)ncomp * g.fplane;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const size_t f = t % g.fplane;
    const int fx = (int)(f % g.fp), fy = (int)(f / g.fp);
    if (fx < 2 || fx >= g.nx + 2 || fy < 2 || fy >= g.ny + 2) v[t] = 0.0;
  }
}
void adj_keep_interior(const Dev2D& d, double* v, int ncomp, cudaStream_t s) {
  k_keep_interior<<<4 * 152, 256, 0, s>>>(d, v, ncomp);
}

void adj_unsort(const Dev2D& d, const Parts64& lA, const Parts64& lB, cudaStream_t s) {
  dim3 grid((d.cap + 255) / 256, d.nrowjob);
  k_adj_unsort<<<grid, 256, 0, s>>>(d, lA, lB, d.map, d.np2new);
}

void adj_particles(const Dev2D& d, const double* luj, const Parts64& lA, const Parts64& lB, double* tmp,
                   double* ltmp, double* luf, float* f32, cudaStream_t s) {
  const size_t n = (size_t)(d.g.nx + 2) * (d.g.ny + 2);
  launch_adj_deposit(d, luj, lA, lB, f32, s);
  k_adj_tmp<<<4 * 152, 256, 0, s>>>(d, tmp);
  cudaMemsetAsync(ltmp, 0, sizeof(double) * 6 * n, s);
  launch_adj_push(d, tmp, lA, lB, ltmp, f32, s);
  k_adj_tmpT<<<4 * 152, 256, 0, s>>>(d, ltmp, luf);
}

// ---- dot-product checks of the transposed linear operators (random vectors) ----
namespace {
__global__ void k_fill_rand(double* v, size_t n, unsigned seed) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const uint4 r = philox4x32(make_uint4((unsigned)i, (unsigned)(i >> 32), seed, 7u), make_uint2(seed, 99u));
    v[i] = u01(r.x, r.y) - 0.5;
  }
}
__global__ void k_dot(const double* a, const double* b, size_t n, double* out) {
  double s = 0.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    s += a[i] * b[i];
  atomicAdd(out, s);
}
}  // namespace

void adj_fill_rand(double* v, size_t n, unsigned seed, cudaStream_t s) { k_fill_rand<<<4 * 152, 256, 0, s>>>(v, n, seed); }
void adj_dot(const double* a, const double* b, size_t n, double* out, cudaStream_t s) {
  k_dot<<<4 * 152, 256, 0, s>>>(a, b, n, out);
}

}  // namespace wpic
