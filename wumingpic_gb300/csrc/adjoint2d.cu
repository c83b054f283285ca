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
// The per-particle Jacobians of the push and the deposit are evaluated in forward mode with
// dual numbers on the same expressions as the forward kernels; the linear field operators
// are transposed by hand (the dot-product identity <L x, y> = <x, L^T y> is checked by
// wpic_adjoint_selfcheck).  Scatters use FP64 atomics: the adjoint is not bitwise
// reproducible, only to round-off.
#include <cmath>

#include "common.cuh"

namespace wpic {

namespace {

// ---- dual numbers: value and N partial derivatives ----
template <int N>
struct Dual {
  double v;
  double d[N];
};

template <int N>
__device__ __forceinline__ Dual<N> dconst(double v) {
  Dual<N> r;
  r.v = v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = 0.0;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> dvar(double v, int k) {
  Dual<N> r = dconst<N>(v);
  r.d[k] = 1.0;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r;
  r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(double s, const Dual<N>& a) {
  Dual<N> r;
  r.v = s * a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = s * a.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator+(double s, const Dual<N>& a) {
  Dual<N> r = a;
  r.v = s + a.v;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  const double ib = 1.0 / b.v;
  r.v = a.v * ib;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> dsqrt(const Dual<N>& a) {
  Dual<N> r;
  r.v = sqrt(a.v);
  const double h = 0.5 / r.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * h;
  return r;
}

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

// ---- the deposit's Jacobian: inputs (x_old, y_old, x_new, y_new, ux', uy', uz') ----
__global__ void k_adj_deposit(Dev2D d, const double* luj, Parts64 lA, Parts64 lB) {
  const Grid2D g = d.g;
  const int row = blockIdx.y;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= d.np2[row]) return;
  const int isp = row / g.ny, jj = row - isp * g.ny;
  const int* ccr = d.cc + (size_t)row * (g.nx + 1);
  const int cx = cell_of(ccr, g.nx, s);
  const size_t k = (size_t)row * d.cap + s;
  const double d_delx = d.ph.d_delx, c = d.ph.c;
  const double qdd = d.ph.q[isp] * d.ph.delx * d.ph.d_delt, fac = 1.0 / 3.0;
  const int iabs = g.nxgs + cx, jabs = g.nygs + jj;
  using D7 = Dual<7>;
  const D7 in[7] = {dvar<7>(d.A.x[k], 0), dvar<7>(d.A.y[k], 1), dvar<7>(d.B.x[k], 2), dvar<7>(d.B.y[k], 3),
                    dvar<7>(d.B.ux[k], 4), dvar<7>(d.B.uy[k], 5), dvar<7>(d.B.uz[k], 6)};
  D7 s0[2][5], ds[2][5];
#pragma unroll
  for (int dim = 0; dim < 2; ++dim) {
    const D7 dh = d_delx * in[dim] + dconst<7>(-0.5 - (double)(dim == 0 ? iabs : jabs));
    s0[dim][0] = dconst<7>(0.0);
    s0[dim][1] = 0.5 * ((0.5 + (-dh)) * (0.5 + (-dh)));
    s0[dim][2] = 0.75 + (-(dh * dh));
    s0[dim][3] = 0.5 * ((0.5 + dh) * (0.5 + dh));
    s0[dim][4] = dconst<7>(0.0);
    const double pnv = in[2 + dim].v;
    const int i2 = (int)(pnv * d_delx);
    const D7 dh1 = d_delx * in[2 + dim] + dconst<7>(-0.5 - (double)i2);
    const int inc = i2 - (dim == 0 ? iabs : jabs);
    const D7 s1_1 = 0.5 * ((0.5 + (-dh1)) * (0.5 + (-dh1)));
    const D7 s1_2 = 0.75 + (-(dh1 * dh1));
    const D7 s1_3 = 0.5 * ((0.5 + dh1) * (0.5 + dh1));
    const int ainc = inc < 0 ? -inc : inc;
    const double m1 = (double)(-(inc - ainc)) * 0.5, m2 = (double)(-ainc + 1), m3 = (double)(inc + ainc) * 0.5;
    ds[dim][0] = m1 * s1_1 - s0[dim][0];
    ds[dim][1] = m2 * s1_1 + m1 * s1_2 - s0[dim][1];
    ds[dim][2] = m2 * s1_2 + m1 * s1_3 + m3 * s1_1 - s0[dim][2];
    ds[dim][3] = m2 * s1_3 + m3 * s1_2 - s0[dim][3];
    ds[dim][4] = m3 * s1_3 - s0[dim][4];
  }
  const D7 u2 = in[4] * in[4] + in[5] * in[5] + in[6] * in[6];
  const D7 gvz = in[6] / dsqrt(1. + (1.0 / (c * c)) * u2);
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  const size_t P = g.fplane;
  auto take = [&](const D7& v, int comp, int a, int b) {  // entry (a, b) of the cell -> node (cx+a, jj+b)
    const double l = luj[(size_t)comp * P + (size_t)(jj + b) * g.fp + (cx + a)];
#pragma unroll
    for (int i = 0; i < 7; ++i) acc[i] += l * v.d[i];
  };
#pragma unroll
  for (int jp = 0; jp < 5; ++jp) {
    const D7 wy = s0[1][jp] + 0.5 * ds[1][jp];
    D7 t = dconst<7>(0.0);
#pragma unroll
    for (int ip = 0; ip < 4; ++ip) {
      t = t - qdd * (ds[0][ip] * wy);
      take(t, 0, ip + 1, jp);
    }
  }
#pragma unroll
  for (int ip = 0; ip < 5; ++ip) {
    const D7 wx = s0[0][ip] + 0.5 * ds[0][ip];
    D7 t = dconst<7>(0.0);
#pragma unroll
    for (int jp = 0; jp < 4; ++jp) {
      t = t - qdd * (ds[1][jp] * wx);
      take(t, 1, ip, jp + 1);
    }
  }
  const D7 qg = d.ph.q[isp] * gvz;
#pragma unroll
  for (int jp = 0; jp < 5; ++jp)
#pragma unroll
    for (int ip = 0; ip < 5; ++ip) {
      const D7 v = qg * (s0[0][ip] * s0[1][jp] + 0.5 * (ds[0][ip] * s0[1][jp]) + 0.5 * (s0[0][ip] * ds[1][jp]) +
                         fac * (ds[0][ip] * ds[1][jp]));
      take(v, 2, ip, jp);
    }
  lA.x[k] += acc[0];
  lA.y[k] += acc[1];
  lB.x[k] += acc[2];
  lB.y[k] += acc[3];
  lB.ux[k] += acc[4];
  lB.uy[k] += acc[5];
  lB.uz[k] += acc[6];
}

// ---- the push's Jacobian: inputs (ux, uy, uz, bpx, bpy, bpz, epx, epy, epz) ----
__global__ void k_adj_push(Dev2D d, const double* tmp, Parts64 lA, Parts64 lB, double* ltmp) {
  const Grid2D g = d.g;
  const int row = blockIdx.y;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= d.np2[row]) return;
  const int isp = row / g.ny, jj = row - isp * g.ny;
  const int* ccr = d.cc + (size_t)row * (g.nx + 1);
  const int cx = cell_of(ccr, g.nx, s);
  const size_t k = (size_t)row * d.cap + s;
  const int tw = g.nx + 2;
  const size_t n = (size_t)tw * (g.ny + 2);
  const double dxi = d.ph.p_d_delx, delt = d.ph.delt, c = d.ph.c;
  const double fac1 = d.ph.q[isp] / d.ph.r[isp] * 0.5 * delt;
  const double txxx = fac1 * fac1;
  const double fac2 = d.ph.q[isp] * delt / d.ph.r[isp];
  const int iabs = g.nxgs + cx, jabs = g.nygs + jj;
  const double x = d.A.x[k], y = d.A.y[k];
  const double hx = x * dxi - 0.5 - (double)iabs, hy = y * dxi - 0.5 - (double)jabs;
  const double sx[3] = {0.5 * (0.5 - hx) * (0.5 - hx), 0.75 - hx * hx, 0.5 * (0.5 + hx) * (0.5 + hx)};
  const double sy[3] = {0.5 * (0.5 - hy) * (0.5 - hy), 0.75 - hy * hy, 0.5 * (0.5 + hy) * (0.5 + hy)};
  const double dsx[3] = {-(0.5 - hx) * dxi, -2.0 * hx * dxi, (0.5 + hx) * dxi};
  const double dsy[3] = {-(0.5 - hy) * dxi, -2.0 * hy * dxi, (0.5 + hy) * dxi};
  // tmp node (a, b) of the particle's cell: local cell (cx - 1 + a, jj - 1 + b) -> index (cx + a, jj + b)
  double fv[6], fdx[6], fdy[6];
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    double v = 0.0, vx = 0.0, vy = 0.0;
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const double t = tmp[(size_t)m * n + (size_t)(jj + b) * tw + (cx + a)];
        v += t * sx[a] * sy[b];
        vx += t * dsx[a] * sy[b];
        vy += t * sx[a] * dsy[b];
      }
    fv[m] = v;
    fdx[m] = vx;
    fdy[m] = vy;
  }
  using D9 = Dual<9>;
  const D9 bpx = dvar<9>(fv[0], 3), bpy = dvar<9>(fv[1], 4), bpz = dvar<9>(fv[2], 5);
  const D9 epx = dvar<9>(fv[3], 6), epy = dvar<9>(fv[4], 7), epz = dvar<9>(fv[5], 8);
  D9 uvm1 = dvar<9>(d.A.ux[k], 0) + fac1 * epx;
  D9 uvm2 = dvar<9>(d.A.uy[k], 1) + fac1 * epy;
  D9 uvm3 = dvar<9>(d.A.uz[k], 2) + fac1 * epz;
  const D9 gam = dsqrt(c * c + (uvm1 * uvm1 + uvm2 * uvm2 + uvm3 * uvm3));
  const D9 igam = dconst<9>(1.0) / gam;
  const D9 fac1r = fac1 * igam;
  const D9 fac2r = dconst<9>(fac2) / (gam + txxx * ((bpx * bpx + bpy * bpy + bpz * bpz) * igam));
  const D9 uvm4 = uvm1 + fac1r * (uvm2 * bpz - uvm3 * bpy);
  const D9 uvm5 = uvm2 + fac1r * (uvm3 * bpx - uvm1 * bpz);
  const D9 uvm6 = uvm3 + fac1r * (uvm1 * bpy - uvm2 * bpx);
  uvm1 = uvm1 + fac2r * (uvm5 * bpz - uvm6 * bpy);
  uvm2 = uvm2 + fac2r * (uvm6 * bpx - uvm4 * bpz);
  uvm3 = uvm3 + fac2r * (uvm4 * bpy - uvm5 * bpx);
  const D9 g3 = uvm1 + fac1 * epx, g4 = uvm2 + fac1 * epy, g5 = uvm3 + fac1 * epz;
  const D9 gi = dconst<9>(1.0) / dsqrt(1.0 + (1.0 / (c * c)) * (g3 * g3 + g4 * g4 + g5 * g5));
  const D9 mx = (delt * g3) * gi, my = (delt * g4) * gi;  // x' - x, y' - y
  const double lx = lB.x[k], ly = lB.y[k], lux = lB.ux[k], luy = lB.uy[k], luz = lB.uz[k];
  double lin[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) lin[i] = lx * mx.d[i] + ly * my.d[i] + lux * g3.d[i] + luy * g4.d[i] + luz * g5.d[i];
  double lxa = lx, lya = ly;
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    lxa += lin[3 + m] * fdx[m];
    lya += lin[3 + m] * fdy[m];
  }
  lA.x[k] += lxa;
  lA.y[k] += lya;
  lA.ux[k] += lin[0];
  lA.uy[k] += lin[1];
  lA.uz[k] += lin[2];
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    const double lf = lin[3 + m];
    if (lf == 0.0) continue;
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int a = 0; a < 3; ++a)
        atomicAdd(ltmp + (size_t)m * n + (size_t)(jj + b) * tw + (cx + a), lf * sx[a] * sy[b]);
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
// the push's field adjoint alone: luf += (dB/duf)^T lB (lA receives the particle part)
void adj_push_fields(const Dev2D& d, const Parts64& lB, const Parts64& lA, double* tmp, double* ltmp, double* luf,
                     cudaStream_t s) {
  const size_t n = (size_t)(d.g.nx + 2) * (d.g.ny + 2);
  k_adj_tmp<<<4 * 152, 256, 0, s>>>(d, tmp);
  cudaMemsetAsync(ltmp, 0, sizeof(double) * 6 * n, s);
  k_adj_push<<<dim3((d.cap + 127) / 128, d.nrowjob), 128, 0, s>>>(d, tmp, lA, lB, ltmp);
  k_adj_tmpT<<<4 * 152, 256, 0, s>>>(d, ltmp, luf);
}

void adj_deposit_only(const Dev2D& d, const double* luj, const Parts64& lA, const Parts64& lB, cudaStream_t s) {
  k_adj_deposit<<<dim3((d.cap + 127) / 128, d.nrowjob), 128, 0, s>>>(d, luj, lA, lB);
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
                   double* ltmp, double* luf, cudaStream_t s) {
  const Grid2D& g = d.g;
  const size_t n = (size_t)(g.nx + 2) * (g.ny + 2);
  dim3 grid((d.cap + 127) / 128, d.nrowjob);
  k_adj_deposit<<<grid, 128, 0, s>>>(d, luj, lA, lB);
  k_adj_tmp<<<4 * 152, 256, 0, s>>>(d, tmp);
  cudaMemsetAsync(ltmp, 0, sizeof(double) * 6 * n, s);
  k_adj_push<<<grid, 128, 0, s>>>(d, tmp, lA, lB, ltmp);
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
