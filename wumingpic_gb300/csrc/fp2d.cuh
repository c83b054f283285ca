// Precision-dependent 2D kernels of the FP64 path.  Included twice, inside
// namespace wpic::exact (compiled with -fmad=false: every operation rounded
// separately, in the reference's evaluation order, so the single-thread
// Fortran results are reproduced bit for bit where no reduction intervenes) and
// inside namespace wpic::fast (FMA contraction allowed; results within a few
// ulp of the exact build).
//
// Requires: wpic_internal.h, common.cuh included before.

// ---------------------------------------------------------------------------
// particle__solv  (2d/common/particle.f90:48-179)
// One CTA per (tile of PUSH_TW cells of a bucket row, species).  The E/B values
// at cell centres, tmp(1:6, i-1:i+1, j-1:j+1) of the reference, are formed once
// per tile in shared memory; every particle of the tile then gathers from there.
// ---------------------------------------------------------------------------
constexpr int PUSH_TW = 32;
constexpr int PUSH_THREADS = 128;

// particle__solv_vay's momentum update (2d/common/particle.f90:182-315; the same in 3D,
// 3d/common/particle.f90:236-419), Vay, Phys. Plasmas 15, 056701 (2008): u' from E and the
// rotation at the old gamma, then the new gamma from Vay's quadratic.  Returns 1/gamma.
__device__ __forceinline__ double vay_update(double fac1, double fac2, double c, double bpx, double bpy, double bpz,
                                             double epx, double epy, double epz, double uvm1, double uvm2, double uvm3,
                                             double* g) {
  double gam = sqrt(c * c + uvm1 * uvm1 + uvm2 * uvm2 + uvm3 * uvm3);
  const double fac1r = fac1 / gam;
  const double uvm4 = uvm1 + fac2 * epx + fac1r * (+uvm2 * bpz - uvm3 * bpy);
  const double uvm5 = uvm2 + fac2 * epy + fac1r * (+uvm3 * bpx - uvm1 * bpz);
  const double uvm6 = uvm3 + fac2 * epz + fac1r * (+uvm1 * bpy - uvm2 * bpx);
  const double taux = fac1 * bpx / c;
  const double tauy = fac1 * bpy / c;
  const double tauz = fac1 * bpz / c;
  const double tau2 = taux * taux + tauy * tauy + tauz * tauz;
  const double ua = (uvm4 * taux + uvm5 * tauy + uvm6 * tauz) / c;
  const double sigma = 1.0 + (uvm4 * uvm4 + uvm5 * uvm5 + uvm6 * uvm6) / (c * c) - tau2;
  const double gam2 = 0.5 * (sigma + sqrt(sigma * sigma + 4.0 * (tau2 + ua * ua)));
  gam = sqrt(gam2);
  const double txxx = 1.0 / (tau2 + gam2);
  g[0] = txxx * (gam2 * uvm4 + c * ua * taux + gam * (uvm5 * tauz - uvm6 * tauy));
  g[1] = txxx * (gam2 * uvm5 + c * ua * tauy + gam * (uvm6 * taux - uvm4 * tauz));
  g[2] = txxx * (gam2 * uvm6 + c * ua * tauz + gam * (uvm4 * tauy - uvm5 * taux));
  return 1.0 / gam;
}

// MODE: PUSH_BORIS = particle__solv, PUSH_VAY = particle__solv_vay, PUSH_MOM = mom_calc__accl
// (2d/common/mom_calc.f90:48-161: the same gather and Boris rotation with the time step
// halved by mom_calc__init (:36); positions copied, no move, IDs not written).
template <int MODE>
__global__ void __launch_bounds__(PUSH_THREADS) k_push2d(Dev2D d) {
  constexpr bool VAY = MODE == PUSH_VAY;
  const Grid2D g = d.g;
  const int c0 = blockIdx.x * PUSH_TW;
  const int jj = blockIdx.y, isp = blockIdx.z;
  if (c0 >= g.nx) return;
  const int nc = min(PUSH_TW, g.nx - c0);
  __shared__ double tmp[6][3][PUSH_TW + 2];
  __shared__ int scc[PUSH_TW + 1];
  const int row = isp * g.ny + jj;
  for (int idx = threadIdx.x; idx < 3 * (nc + 2); idx += blockDim.x) {
    const int rj = idx / (nc + 2), ci = idx - rj * (nc + 2);
    const int fi = c0 + ci + 1, fj = jj + rj + 1;  // field index of cell (c0+ci-1, jj+rj-1)
    const double* U = d.uf;
    const size_t b0 = (size_t)fj * g.fp + fi;
#define UF(c, di, dj) U[(size_t)(c) * g.fplane + b0 + (size_t)(dj) * g.fp + (di)]
    tmp[0][rj][ci] = 0.5 * (+UF(0, 0, 0) + UF(0, 0, 1));
    tmp[1][rj][ci] = 0.5 * (+UF(1, 0, 0) + UF(1, 1, 0));
    tmp[2][rj][ci] = 0.25 * (+UF(2, 0, 0) + UF(2, 1, 0) + UF(2, 0, 1) + UF(2, 1, 1));
    tmp[3][rj][ci] = 0.5 * (+UF(3, 0, 0) + UF(3, 1, 0));
    tmp[4][rj][ci] = 0.5 * (+UF(4, 0, 0) + UF(4, 0, 1));
    tmp[5][rj][ci] = UF(5, 0, 0);
#undef UF
  }
  for (int idx = threadIdx.x; idx <= nc; idx += blockDim.x) scc[idx] = d.cc[(size_t)row * (g.nx + 1) + c0 + idx];
  __syncthreads();

  const double dxi = d.ph.p_d_delx, delt = MODE == PUSH_MOM ? d.ph.delt * 0.5 : d.ph.delt, c = d.ph.c;
  const double fac1 = d.ph.q[isp] / d.ph.r[isp] * 0.5 * delt;
  const double txxx = fac1 * fac1;
  const double fac2 = d.ph.q[isp] * delt / d.ph.r[isp];
#if !WPIC_REF_ORDER
  const double ic2 = 1.0 / (c * c);
#endif
  const int jabs = g.nygs + jj;
  const size_t rbase = (size_t)row * d.cap;
  const int s_end = scc[nc];
  for (int s = scc[0] + threadIdx.x; s < s_end; s += blockDim.x) {
    int lo = 0, hi = nc;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (scc[mid] <= s) lo = mid; else hi = mid;
    }
    const int iabs = g.nxgs + c0 + lo;
    const size_t k = rbase + s;
    const double x = d.A.x[k], y = d.A.y[k];
    double dh = x * dxi - 0.5 - (double)iabs;
    const double sx0 = 0.5 * (0.5 - dh) * (0.5 - dh);
    const double sx1 = 0.75 - dh * dh;
    const double sx2 = 0.5 * (0.5 + dh) * (0.5 + dh);
    dh = y * dxi - 0.5 - (double)jabs;
    const double sy0 = 0.5 * (0.5 - dh) * (0.5 - dh);
    const double sy1 = 0.75 - dh * dh;
    const double sy2 = 0.5 * (0.5 + dh) * (0.5 + dh);
    double f[6];
#if WPIC_REF_ORDER
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      f[m] = +(+tmp[m][0][lo] * sx0 + tmp[m][0][lo + 1] * sx1 + tmp[m][0][lo + 2] * sx2) * sy0
             + (+tmp[m][1][lo] * sx0 + tmp[m][1][lo + 1] * sx1 + tmp[m][1][lo + 2] * sx2) * sy1
             + (+tmp[m][2][lo] * sx0 + tmp[m][2][lo + 1] * sx1 + tmp[m][2][lo + 2] * sx2) * sy2;
    }
#else
    // FMA build: the nine node weights once, then nine fused multiply-adds per component
    // (63 FP64 instructions for the gather instead of 72; the FP64 pipe is the bound)
    {
      const double wx[3] = {sx0, sx1, sx2}, wy[3] = {sy0, sy1, sy2};
      double w[3][3];
#pragma unroll
      for (int rj = 0; rj < 3; ++rj)
#pragma unroll
        for (int ci = 0; ci < 3; ++ci) w[rj][ci] = wy[rj] * wx[ci];
#pragma unroll
      for (int m = 0; m < 6; ++m) {
        double v = tmp[m][0][lo] * w[0][0];
#pragma unroll
        for (int q = 1; q < 9; ++q) v = fma(tmp[m][q / 3][lo + q % 3], w[q / 3][q % 3], v);
        f[m] = v;
      }
    }
#endif
    const double bpx = f[0], bpy = f[1], bpz = f[2], epx = f[3], epy = f[4], epz = f[5];
    if (VAY) {
      double gv[3];
      const double ig = vay_update(fac1, fac2, c, bpx, bpy, bpz, epx, epy, epz, d.A.ux[k], d.A.uy[k], d.A.uz[k], gv);
      d.B.ux[k] = gv[0];
      d.B.uy[k] = gv[1];
      d.B.uz[k] = gv[2];
      d.B.x[k] = x + gv[0] * delt * ig;
      d.B.y[k] = y + gv[1] * delt * ig;
      d.B.id[k] = d.A.id[k];
      continue;
    }
    double uvm1 = d.A.ux[k] + fac1 * epx;
    double uvm2 = d.A.uy[k] + fac1 * epy;
    double uvm3 = d.A.uz[k] + fac1 * epz;
#if WPIC_REF_ORDER
    double gam = sqrt(c * c + uvm1 * uvm1 + uvm2 * uvm2 + uvm3 * uvm3);
    const double igam = 1. / gam;
#else
    // FMA build: one reciprocal square root gives 1/gamma and gamma (the reference takes a
    // square root and then divides); 1/c^2 once per thread
    const double gsq = c * c + uvm1 * uvm1 + uvm2 * uvm2 + uvm3 * uvm3;
    const double igam = rsqrt(gsq);
    double gam = gsq * igam;
#endif
    const double fac1r = fac1 * igam;
    const double fac2r = fac2 / (gam + txxx * (bpx * bpx + bpy * bpy + bpz * bpz) * igam);
    const double uvm4 = uvm1 + fac1r * (+uvm2 * bpz - uvm3 * bpy);
    const double uvm5 = uvm2 + fac1r * (+uvm3 * bpx - uvm1 * bpz);
    const double uvm6 = uvm3 + fac1r * (+uvm1 * bpy - uvm2 * bpx);
    uvm1 = uvm1 + fac2r * (+uvm5 * bpz - uvm6 * bpy);
    uvm2 = uvm2 + fac2r * (+uvm6 * bpx - uvm4 * bpz);
    uvm3 = uvm3 + fac2r * (+uvm4 * bpy - uvm5 * bpx);
    const double g3 = uvm1 + fac1 * epx;
    const double g4 = uvm2 + fac1 * epy;
    const double g5 = uvm3 + fac1 * epz;
    if (MODE == PUSH_MOM) {
      d.B.x[k] = x;
      d.B.y[k] = y;
      d.B.ux[k] = g3;
      d.B.uy[k] = g4;
      d.B.uz[k] = g5;
      continue;
    }
#if WPIC_REF_ORDER
    gam = 1.0 / sqrt(1.0 + (+g3 * g3 + g4 * g4 + g5 * g5) / (c * c));
#else
    gam = rsqrt(1.0 + (g3 * g3 + g4 * g4 + g5 * g5) * ic2);
#endif
    d.B.ux[k] = g3;
    d.B.uy[k] = g4;
    d.B.uz[k] = g5;
    d.B.x[k] = x + g3 * delt * gam;
    d.B.y[k] = y + g4 * delt * gam;
    d.B.id[k] = d.A.id[k];
  }
}

void push2d(const Dev2D& d, cudaStream_t s) {
  dim3 grid((d.g.nx + PUSH_TW - 1) / PUSH_TW, d.g.ny, d.ph.nsp);
  k_push2d<PUSH_BORIS><<<grid, PUSH_THREADS, 0, s>>>(d);
}

void push_vay2d(const Dev2D& d, cudaStream_t s) {
  dim3 grid((d.g.nx + PUSH_TW - 1) / PUSH_TW, d.g.ny, d.ph.nsp);
  k_push2d<PUSH_VAY><<<grid, PUSH_THREADS, 0, s>>>(d);
}

void mom_accl2d(const Dev2D& d, cudaStream_t s) {
  dim3 grid((d.g.nx + PUSH_TW - 1) / PUSH_TW, d.g.ny, d.ph.nsp);
  k_push2d<PUSH_MOM><<<grid, PUSH_THREADS, 0, s>>>(d);
}

// ---------------------------------------------------------------------------
// mom_calc__nvt  (2d/common/mom_calc.f90:164-249)
// One thread per node (I, J) of mom(7, nxgs-1:nxge+1, nys-1:nye+1, nsp).  A node takes
// contributions only from particles of cells I-1..I+1 in rows J-1..J+1; the thread walks
// those rows in ascending j and, within a row, the three cells' particles in storage
// order, so every node is the single-thread reference's sum (0 + c1) + c2 + ... .  The
// cells come from cumcnt, so the particles must be bucket-sorted (up after sort__bucket,
// or gp after mom_calc__accl); a particle outside the 2x2 node stencil of its cell is
// reported as out of range instead of being dropped.
// ---------------------------------------------------------------------------
constexpr int MOM_TX = 128;

__global__ void __launch_bounds__(MOM_TX) k_mom_nvt2d(Dev2D d, Parts64 P, double* mom) {
  const Grid2D g = d.g;
  const int nxm = g.nx + 2;
  const int in = blockIdx.x * MOM_TX + threadIdx.x, jn = blockIdx.y, isp = blockIdx.z;
  if (in >= nxm) return;
  const int I = g.nxgs - 1 + in, J = g.nygs - 1 + jn;
  const double d_delx = d.ph.d_delx, c = d.ph.c;
  double acc[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  bool bad = false;
  for (int dj = -1; dj <= 1; ++dj) {
    const int jj = jn - 1 + dj;  // particle row J + dj
    if (jj < 0 || jj >= g.ny) continue;
    const int row = isp * g.ny + jj;
    const int* ccr = d.cc + (size_t)row * (g.nx + 1);
    const int c_lo = max(in - 2, 0), c_hi = min(in, g.nx - 1);  // cells I-1..I+1
    if (c_lo > c_hi) continue;
    const int s0 = ccr[c_lo], s1 = ccr[c_hi + 1];
    // the cell with the node's own index is checked by this thread (row J only)
    const int own0 = (dj == 0 && in >= 1 && in <= g.nx) ? ccr[in - 1] : 0;
    const int own1 = (dj == 0 && in >= 1 && in <= g.nx) ? ccr[in] : 0;
    const size_t rbase = (size_t)row * d.cap;
    for (int s = s0; s < s1; ++s) {
      const size_t k = rbase + s;
      const double x = P.x[k], y = P.y[k];
      const int ih = (int)(x * d_delx - 0.5);
      const int jh = (int)(y * d_delx - 0.5);
      if (s >= own0 && s < own1 && (ih < I - 1 || ih > I || jh < J - 1 || jh > J)) bad = true;
      const int a = I - ih, b = J - jh;
      if (a < 0 || a > 1 || b < 0 || b > 1) continue;
      const double dx = x * d_delx - 0.5 - ih, dxm = 1. - dx;
      const double dy = y * d_delx - 0.5 - jh, dym = 1. - dy;
      const double wx = a ? dx : dxm, wy = b ? dy : dym;
      const double u1 = P.ux[k], u2 = P.uy[k], u3 = P.uz[k];
      const double gam = 1. / sqrt(1.0 + (+u1 * u1 + u2 * u2 + u3 * u3) / (c * c));
      acc[0] = acc[0] + wx * wy;
      acc[1] = acc[1] + u1 * gam * wx * wy;
      acc[2] = acc[2] + u2 * gam * wx * wy;
      acc[3] = acc[3] + u3 * gam * wx * wy;
      acc[4] = acc[4] + u1 * u1 * gam * wx * wy;
      acc[5] = acc[5] + u2 * u2 * gam * wx * wy;
      acc[6] = acc[6] + u3 * u3 * gam * wx * wy;
    }
  }
  if (bad) atomicOr(d.err, EB_OUT_OF_RANGE);
  double* o = mom + 7 * ((size_t)in + (size_t)nxm * ((size_t)jn + (size_t)(g.ny + 2) * isp));
#pragma unroll
  for (int l = 0; l < 7; ++l) o[l] = acc[l];
}

#if !WPIC_REF_ORDER
// The FMA build sums the same moments without the reference's summation order (within 1e-12):
// one thread per cell walks its particles once, each particle's seven moments added into the
// cell's 3 x 3 node tile (the particle's 2 x 2 nodes start at node column cx or cx + 1 and row
// jj or jj + 1), and a second kernel adds the nine tiles that touch each node.  The tiles of
// one species at a time go to the deposit's cell buffer (63 of its 75 planes).
constexpr int MOMC_T = 64;

__global__ void __launch_bounds__(MOMC_T) k_mom_cell2d(Dev2D d, Parts64 P, int isp) {
  extern __shared__ double macc[];  // [63][MOMC_T]: moment l of tile node (ta, tb) at l + 7 (ta + 3 tb)
  const Grid2D g = d.g;
  const int cx = blockIdx.x * MOMC_T + threadIdx.x, jj = blockIdx.y;
  if (cx >= g.nx) return;
  double* a = macc + threadIdx.x;
#pragma unroll 7
  for (int e = 0; e < 63; ++e) a[e * MOMC_T] = 0.0;
  const double d_delx = d.ph.d_delx, c = d.ph.c, ic2 = 1.0 / (c * c);
  const int row = isp * g.ny + jj;
  const int* ccr = d.cc + (size_t)row * (g.nx + 1);
  const int i0 = g.nxgs - 1 + cx, j0 = g.nygs - 1 + jj;  // indices of tile node (0, 0)
  const size_t rbase = (size_t)row * d.cap;
  bool bad = false;
  for (int sl = ccr[cx]; sl < ccr[cx + 1]; ++sl) {
    const size_t k = rbase + sl;
    const double x = P.x[k], y = P.y[k];
    const int ih = (int)(x * d_delx - 0.5), jh = (int)(y * d_delx - 0.5);
    const int ta = ih - i0, tb = jh - j0;
    if (ta < 0 || ta > 1 || tb < 0 || tb > 1) {
      bad = true;
      continue;
    }
    const double dx = x * d_delx - 0.5 - ih, dy = y * d_delx - 0.5 - jh;
    const double u1 = P.ux[k], u2 = P.uy[k], u3 = P.uz[k];
    const double gam = 1. / sqrt(1.0 + (u1 * u1 + u2 * u2 + u3 * u3) * ic2);
    const double pre[7] = {1.0, u1 * gam, u2 * gam, u3 * gam, u1 * u1 * gam, u2 * u2 * gam, u3 * u3 * gam};
    const double wx[2] = {1. - dx, dx}, wy[2] = {1. - dy, dy};
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int aa = 0; aa < 2; ++aa) {
        const double w = wx[aa] * wy[b];
        double* t = a + 7 * ((ta + aa) + 3 * (tb + b)) * MOMC_T;
#pragma unroll
        for (int l = 0; l < 7; ++l) t[l * MOMC_T] = fma(pre[l], w, t[l * MOMC_T]);
      }
  }
  if (bad) atomicOr(d.err, EB_OUT_OF_RANGE);
  const size_t cell = (size_t)jj * g.nx + cx;
#pragma unroll 7
  for (int e = 0; e < 63; ++e) d.cellJ[(size_t)e * g.ncell + cell] = a[e * MOMC_T];
}

// node (in, jn) of species isp: the tiles of cells in-2..in, jn-2..jn
__global__ void k_mom_gather2d(Dev2D d, double* mom, int isp) {
  const Grid2D g = d.g;
  const int nxm = g.nx + 2;
  const int in = blockIdx.x * blockDim.x + threadIdx.x, jn = blockIdx.y;
  if (in >= nxm) return;
  double acc[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int tb = 0; tb < 3; ++tb) {
    const int jj = jn - tb;
    if (jj < 0 || jj >= g.ny) continue;
    for (int ta = 0; ta < 3; ++ta) {
      const int cx = in - ta;
      if (cx < 0 || cx >= g.nx) continue;
      const size_t cell = (size_t)jj * g.nx + cx;
#pragma unroll
      for (int l = 0; l < 7; ++l) acc[l] += d.cellJ[(size_t)(l + 7 * (ta + 3 * tb)) * g.ncell + cell];
    }
  }
  double* o = mom + 7 * ((size_t)in + (size_t)nxm * ((size_t)jn + (size_t)(g.ny + 2) * isp));
#pragma unroll
  for (int l = 0; l < 7; ++l) o[l] = acc[l];
}
#endif

void mom_nvt2d(const Dev2D& d, const Parts64& P, double* mom, cudaStream_t s) {
#if WPIC_REF_ORDER
  dim3 grid((d.g.nx + 2 + MOM_TX - 1) / MOM_TX, d.g.ny + 2, d.ph.nsp);
  k_mom_nvt2d<<<grid, MOM_TX, 0, s>>>(d, P, mom);
#else
  for (int isp = 0; isp < d.ph.nsp; ++isp) {
    k_mom_cell2d<<<dim3((d.g.nx + MOMC_T - 1) / MOMC_T, d.g.ny), MOMC_T, 63 * MOMC_T * sizeof(double), s>>>(d, P, isp);
    k_mom_gather2d<<<dim3((d.g.nx + 2 + 127) / 128, d.g.ny + 2), 128, 0, s>>>(d, mom, isp);
  }
#endif
}

// ---------------------------------------------------------------------------
// ele_cur  (2d/common/field.f90:189-316)
// One thread per cell walks the cell's particles of both species in bucket
// order and accumulates the cell's 5x5 Esirkepov tiles pjx/pjy/pjz exactly as
// the reference does (shared memory, one column per thread); the tiles go to
// cellJ and k_jgather2d adds them into uj in the reference's (j, i) cell order,
// which is the single-thread OpenMP reduction order.
// ---------------------------------------------------------------------------
constexpr int DEP_THREADS = 64;

__global__ void __launch_bounds__(DEP_THREADS) k_deposit2d(Dev2D d) {
  extern __shared__ double acc[];  // [75][DEP_THREADS]: pjx(ip,jp) at (ip+2)+5*(jp+2), pjy at 25+, pjz at 50+
  const Grid2D g = d.g;
  const int cx = blockIdx.x * DEP_THREADS + threadIdx.x;
  const int jj = blockIdx.y;
  if (cx >= g.nx) return;
  double* a = acc + threadIdx.x;
#pragma unroll 5
  for (int e = 0; e < 75; ++e) a[e * DEP_THREADS] = 0.0;
  const double d_delx = d.ph.d_delx, d_delt = d.ph.d_delt, delx = d.ph.delx, c = d.ph.c;
  const double fac = 1.0 / 3.0;
#if !WPIC_REF_ORDER
  const double ic2 = 1.0 / (c * c);
#endif
  const int iabs = g.nxgs + cx, jabs = g.nygs + jj;
  for (int isp = 0; isp < d.ph.nsp; ++isp) {
    const int row = isp * g.ny + jj;
    const int* ccr = d.cc + (size_t)row * (g.nx + 1);
    const int s0i = ccr[cx], s1i = ccr[cx + 1];
    const double qs = d.ph.q[isp];
    const double qdd = qs * delx * d_delt;
    const size_t rbase = (size_t)row * d.cap;
    for (int s = s0i; s < s1i; ++s) {
      const size_t k = rbase + s;
      double s0x[5], s0y[5], dsx[5], dsy[5];
      double dh = d.A.x[k] * d_delx - 0.5 - (double)iabs;
      s0x[0] = 0.0;
      s0x[1] = 0.5 * (0.5 - dh) * (0.5 - dh);
      s0x[2] = 0.75 - dh * dh;
      s0x[3] = 0.5 * (0.5 + dh) * (0.5 + dh);
      s0x[4] = 0.0;
      dh = d.A.y[k] * d_delx - 0.5 - (double)jabs;
      s0y[0] = 0.0;
      s0y[1] = 0.5 * (0.5 - dh) * (0.5 - dh);
      s0y[2] = 0.75 - dh * dh;
      s0y[3] = 0.5 * (0.5 + dh) * (0.5 + dh);
      s0y[4] = 0.0;
      const double xn = d.B.x[k], yn = d.B.y[k];
#pragma unroll
      for (int dim = 0; dim < 2; ++dim) {
        const double pn = dim == 0 ? xn : yn;
        const int i2 = (int)(pn * d_delx);
        const double dh1 = pn * d_delx - 0.5 - (double)i2;
        const int inc = i2 - (dim == 0 ? iabs : jabs);
        if (inc < -1 || inc > 1) atomicOr(d.err, EB_MOVED_TOO_FAR);
        const double s1_1 = 0.5 * (0.5 - dh1) * (0.5 - dh1);
        const double s1_2 = 0.75 - dh1 * dh1;
        const double s1_3 = 0.5 * (0.5 + dh1) * (0.5 + dh1);
        const int ainc = inc < 0 ? -inc : inc;
        const double smo_1 = (double)(-(inc - ainc)) * 0.5;
        const double smo_2 = (double)(-ainc + 1);
        const double smo_3 = (double)(inc + ainc) * 0.5;
        double* ds = dim == 0 ? dsx : dsy;
        const double* s0 = dim == 0 ? s0x : s0y;
        ds[0] = s1_1 * smo_1 - s0[0];
        ds[1] = s1_1 * smo_2 + s1_2 * smo_1 - s0[1];
        ds[2] = s1_2 * smo_2 + s1_3 * smo_1 + s1_1 * smo_3 - s0[2];
        ds[3] = s1_3 * smo_2 + s1_2 * smo_3 - s0[3];
        ds[4] = s1_3 * smo_3 - s0[4];
      }
      const double g3 = d.B.ux[k], g4 = d.B.uy[k], g5 = d.B.uz[k];
#if WPIC_REF_ORDER
      const double gvz = g5 / sqrt(1. + (+g3 * g3 + g4 * g4 + g5 * g5) / (c * c));
#else
      const double gvz = g5 * rsqrt(1. + (g3 * g3 + g4 * g4 + g5 * g5) * ic2);
#endif
#if !WPIC_REF_ORDER
      // The same sums in factored form: the weights q dx/dt (s0 + ds/2) and q vz (s0_y + ds_y/2),
      // q vz (s0_y/2 + ds_y/3) once per row or column; the prefix sums of ds_x and ds_y once per
      // particle, so that every pjx / pjy entry is one fused multiply-add into its accumulator;
      // pjz = s0_x (x) A_y + ds_x (x) B_y as two fused multiply-adds into the accumulator, the
      // zero entries of s0_x left out.  About 190 FP64 instructions per particle; the pipe is
      // the bound (GB300 issues FP64 at 1/64 of the FP32 rate).
      {
        const double qg = qs * gvz;
        double qwy[5], qwx[5], qay[5], qby[5];
#pragma unroll
        for (int e = 0; e < 5; ++e) {
          const double wy = s0y[e] + 0.5 * dsy[e];
          qwy[e] = qdd * wy;
          qay[e] = qg * wy;
          qby[e] = qg * (0.5 * s0y[e] + fac * dsy[e]);
          qwx[e] = qdd * (s0x[e] + 0.5 * dsx[e]);
        }
        double px[4], py[4];
        px[0] = dsx[0];
        py[0] = dsy[0];
#pragma unroll
        for (int q = 1; q < 4; ++q) {
          px[q] = px[q - 1] + dsx[q];
          py[q] = py[q - 1] + dsy[q];
        }
#pragma unroll
        for (int jp = 0; jp < 5; ++jp)
#pragma unroll
          for (int ip = 0; ip < 4; ++ip) {
            double* e = a + ((ip + 1) + 5 * jp) * DEP_THREADS;
            *e = fma(-px[ip], qwy[jp], *e);
          }
#pragma unroll
        for (int ip = 0; ip < 5; ++ip)
#pragma unroll
          for (int jp = 0; jp < 4; ++jp) {
            double* e = a + (25 + ip + 5 * (jp + 1)) * DEP_THREADS;
            *e = fma(-py[jp], qwx[ip], *e);
          }
#pragma unroll
        for (int jp = 0; jp < 5; ++jp)
#pragma unroll
          for (int ip = 0; ip < 5; ++ip) {
            double* e = a + (50 + ip + 5 * jp) * DEP_THREADS;
            double v = fma(dsx[ip], qby[jp], *e);
            if (ip != 0 && ip != 4) v = fma(s0x[ip], qay[jp], v);
            *e = v;
          }
      }
#else
      // pjx: prefix along x, pjtmp(ip+1,jp) = pjtmp(ip,jp) - q*delx/dt*ds_x(ip)*(s0_y(jp)+ds_y(jp)/2)
#pragma unroll
      for (int jp = 0; jp < 5; ++jp) {
        const double wy = s0y[jp] + 0.5 * dsy[jp];
        double t = 0.0;
#pragma unroll
        for (int ip = 0; ip < 4; ++ip) {
          t = t - qdd * dsx[ip] * wy;
          double* e = a + ((ip + 1) + 5 * jp) * DEP_THREADS;
          *e = *e + t;
        }
      }
      // pjy: prefix along y
#pragma unroll
      for (int ip = 0; ip < 5; ++ip) {
        const double wx = s0x[ip] + 0.5 * dsx[ip];
        double t = 0.0;
#pragma unroll
        for (int jp = 0; jp < 4; ++jp) {
          t = t - qdd * dsy[jp] * wx;
          double* e = a + (25 + ip + 5 * (jp + 1)) * DEP_THREADS;
          *e = *e + t;
        }
      }
      // pjz: out-of-plane current with the 1/3 cross term
      const double qg = qs * gvz;
#pragma unroll
      for (int jp = 0; jp < 5; ++jp) {
#pragma unroll
        for (int ip = 0; ip < 5; ++ip) {
          double* e = a + (50 + ip + 5 * jp) * DEP_THREADS;
          *e = *e + qg * (+s0x[ip] * s0y[jp] + 0.5 * dsx[ip] * s0y[jp] + 0.5 * s0x[ip] * dsy[jp]
                          + fac * dsx[ip] * dsy[jp]);
        }
      }
#endif
    }
  }
  const size_t cell = (size_t)jj * g.nx + cx;
#pragma unroll 5
  for (int e = 0; e < 75; ++e) d.cellJ[(size_t)e * g.ncell + cell] = a[e * DEP_THREADS];
}

// uj(node) = sum over the 25 neighbouring cells, in the reference's cell loop
// order (j ascending, then i ascending), of that cell's tile entry.
__global__ void k_jgather2d(Dev2D d) {
  const Grid2D g = d.g;
  const int ii = blockIdx.x * blockDim.x + threadIdx.x;  // field column 0..nx+3
  const int jf = blockIdx.y;                              // field row 0..ny+3
  if (ii >= g.nx + 4) return;
  double sx = 0.0, sy = 0.0, sz = 0.0;
  for (int jp = 2; jp >= -2; --jp) {
    const int cy = jf - 2 - jp;
    if (cy < 0 || cy >= g.ny) continue;
    for (int ip = 2; ip >= -2; --ip) {
      const int cx = ii - 2 - ip;
      if (cx < 0 || cx >= g.nx) continue;
      const size_t cell = (size_t)cy * g.nx + cx;
      const int e = (ip + 2) + 5 * (jp + 2);
      sx = sx + d.cellJ[(size_t)e * g.ncell + cell];
      sy = sy + d.cellJ[(size_t)(25 + e) * g.ncell + cell];
      sz = sz + d.cellJ[(size_t)(50 + e) * g.ncell + cell];
    }
  }
  const size_t f = (size_t)jf * g.fp + ii;
  d.uj[f] = sx;
  d.uj[(size_t)g.fplane + f] = sy;
  d.uj[2 * (size_t)g.fplane + f] = sz;
}

void deposit2d(const Dev2D& d, cudaStream_t s) {
  dim3 grid((d.g.nx + DEP_THREADS - 1) / DEP_THREADS, d.g.ny);
  const size_t shm = (size_t)75 * DEP_THREADS * sizeof(double);
  k_deposit2d<<<grid, DEP_THREADS, shm, s>>>(d);
  dim3 g2((d.g.nx + 4 + 127) / 128, d.g.ny + 4);
  k_jgather2d<<<g2, 128, 0, s>>>(d);
}

// ---------------------------------------------------------------------------
// RHS gkl of the implicit B solve  (2d/common/field.f90:125-146)
// ---------------------------------------------------------------------------
__global__ void k_gkl2d(Dev2D d) {
  const Grid2D g = d.g;
  const int cx = blockIdx.x * blockDim.x + threadIdx.x, cy = blockIdx.y;
  if (cx < g.wx0 || cx > g.wx1) return;  // the active window nxs..nxe
  const size_t f = (size_t)(cy + 2) * g.fp + (cx + 2);
  const size_t P = g.fplane;
  const double* uf = d.uf;
  const double* uj = d.uj;
  const double f1 = d.ph.f1, f2 = d.ph.f2, f3 = d.ph.f3;
  const size_t S = f - g.fp, W = f - 1, E = f + 1, N = f + g.fp;
#define U(c, at) uf[(c) * P + (at)]
#define J(c, at) uj[(c) * P + (at)]
  const double g1 = +f2 * (+U(0, S) + U(0, W) - 4. * U(0, f) + U(0, E) + U(0, N) + f3 * (-J(2, S) + J(2, f)))
                    - f1 * (-U(5, S) + U(5, f));
  const double g2 = +f2 * (+U(1, S) + U(1, W) - 4. * U(1, f) + U(1, E) + U(1, N) - f3 * (-J(2, W) + J(2, f)))
                    + f1 * (-U(5, W) + U(5, f));
  const double g3 = +f2 * (+U(2, S) + U(2, W) - 4. * U(2, f) + U(2, E) + U(2, N)
                           + f3 * (-J(1, W) + J(1, f) + J(0, S) - J(0, f)))
                    - f1 * (-U(4, W) + U(4, f) + U(3, S) - U(3, f));
#undef U
#undef J
  const size_t c = (size_t)cy * g.nx + cx;
  d.gkl[c] = g1;
  d.gkl[(size_t)g.ncell + c] = g2;
  d.gkl[2 * (size_t)g.ncell + c] = g3;
}

void gkl2d(const Dev2D& d, cudaStream_t s) {
  dim3 grid((d.g.nx + 127) / 128, d.g.ny);
  k_gkl2d<<<grid, 128, 0, s>>>(d);
}

// ---------------------------------------------------------------------------
// cgm  (2d/common/field.f90:319-461), the three components solved side by side
// (blockIdx.y = component).  Dot products are reduced deterministically: fixed
// per-block tree, then a fixed-order sum of the block partials.  The stopping
// rule is the reference's, quirks included: the first loop test compares
// ||b||^2 with eps, and ||r|| is taken before the update, so one extra
// iteration runs after convergence.
// ---------------------------------------------------------------------------
constexpr int CG_THREADS = 256;

// The boundary_*__phi ghost rules as index arithmetic on the window nxs..nxe (cells wx0..wx1):
// periodic y; x periodic, conducting walls (boundary_reconnection__phi,
// 2d/proj/reconnection/boundary_reconnection.f90:505-579) or the shock's wall and zero
// right end (boundary_shock__phi, 2d/proj/shock/boundary_shock.f90:551-625).  Returns the
// source cell of (cx, cy) with the sign flag, or cx = -1 where the ghost value is zero.
// The sign flip is an integer flag so that no FP64 compare is issued.
__device__ __forceinline__ void phi_src(const Grid2D& g, int bc, int l, int& cx, int& cy, bool& neg) {
  if (cy < 0) cy += g.ny; else if (cy >= g.ny) cy -= g.ny;
  neg = false;
  if (cx < g.wx0) {
    if (bc == BC_PERIODIC) cx += g.nx;
    else if (l == 0) { cx = g.wx0; neg = true; }
    else cx = g.wx0 + 1;
  } else if (cx > g.wx1) {
    if (bc == BC_PERIODIC) cx -= g.nx;
    else if (bc == BC_SHOCK) cx = -1;
    else if (l == 0) { cx = g.wx1 - 2; neg = true; }
    else cx = g.wx1 - 1;
  }
}

// x or -x by flipping the sign bit with an integer XOR: the conditional negation would
// otherwise cost an FP64 instruction, and the CG stencils are FP64-pipe bound (GB300 runs
// FP64 at 1/64 of FP32)
__device__ __forceinline__ double flip_sign(double x, bool neg) {
  return __longlong_as_double(__double_as_longlong(x) ^ ((long long)neg << 63));
}

__device__ __forceinline__ double phi_at(const double* v, const Grid2D& g, int bc, int l, int cx, int cy) {
  bool neg;
  phi_src(g, bc, l, cx, cy, neg);
  if (cx < 0) return 0.0;
  return flip_sign(v[(size_t)cy * g.nx + cx], neg);
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int w = CG_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + w];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

// phase 0: phi = db(l), b = f5*gkl(l), r = b + N(phi) - f4 phi, p = r; partials of b.b and r.r
__global__ void __launch_bounds__(CG_THREADS) k_cg_init(Dev2D d) {
  __shared__ double sh[CG_THREADS];
  const Grid2D g = d.g;
  const int l = blockIdx.y;
  const size_t off = (size_t)l * g.ncell;
  const double f4 = d.ph.f4, f5 = d.ph.f5;
  double sb = 0.0, sr = 0.0;
  for (int c = blockIdx.x * CG_THREADS + threadIdx.x; c < g.ncell; c += gridDim.x * CG_THREADS) {
    const int cy = c / g.nx, cx = c - cy * g.nx;
    if (cx < g.wx0 || cx > g.wx1) continue;  // outside the window: not part of the system
    // db interior viewed as a [ny][nx] array with pitch fp
    const double* db = d.df + (size_t)l * g.fplane + 2 * (size_t)g.fp + 2;
    auto ph = [&](int x, int y) {
      bool neg;
      phi_src(g, d.ph.bc, l, x, y, neg);
      if (x < 0) return 0.0;
      return flip_sign(db[(size_t)y * g.fp + x], neg);
    };
    const double pc = ph(cx, cy);
    const double b = f5 * d.gkl[off + c];
    const double r = b + ph(cx, cy - 1) + ph(cx - 1, cy) - f4 * pc + ph(cx + 1, cy) + ph(cx, cy + 1);
    d.phi[off + c] = pc;
    d.b[off + c] = b;
    d.r[off + c] = r;
    d.p[off + c] = r;
    sb = sb + b * b;
    sr = sr + r * r;
  }
  sb = block_sum(sb, sh);
  sr = block_sum(sr, sh);
  if (threadIdx.x == 0) {
    d.partials[((size_t)l * d.nred + blockIdx.x) * 2 + 0] = sb;
    d.partials[((size_t)l * d.nred + blockIdx.x) * 2 + 1] = sr;
  }
}

__device__ __forceinline__ void final_sums(const Dev2D& d, int l, double* sh, double* out0, double* out1) {
  double a = 0.0, b = 0.0;
  for (int k = threadIdx.x; k < d.nred; k += CG_THREADS) {
    a = a + d.partials[((size_t)l * d.nred + k) * 2 + 0];
    b = b + d.partials[((size_t)l * d.nred + k) * 2 + 1];
  }
  a = block_sum(a, sh);
  b = block_sum(b, sh);
  *out0 = a;
  *out1 = b;
}

__global__ void __launch_bounds__(CG_THREADS) k_cg_init_fin(Dev2D d) {
  __shared__ double sh[CG_THREADS];
  const int l = blockIdx.x;
  double sb, sr;
  final_sums(d, l, sh, &sb, &sr);
  if (threadIdx.x == 0) {
    CGState& st = d.cg[l];
    st.sum_g = sb;
    st.eps = sqrt(sb) * d.cg_rtol;
    st.sumr_g = sr;
    st.ite = 0;
    if (st.fixed >= 0) st.active = st.fixed > 0;
    else st.active = (sqrt(sr) > st.eps) && (st.sum_g > st.eps);
  }
}

// ap = (f4 - N) p ; partial of p.ap.  The reference also sums r.r here (field.f90:403);
// r has not changed since the previous iteration's r.r (or the initial one), which was
// reduced in this same deterministic order, so that sum is carried instead of recomputed.
__global__ void __launch_bounds__(CG_THREADS) k_cg_ap(Dev2D d) {
  __shared__ double sh[CG_THREADS];
  const Grid2D g = d.g;
  const int l = blockIdx.y;
  if (!d.cg[l].active) return;
  const size_t off = (size_t)l * g.ncell;
  const double f4 = d.ph.f4;
  const double* p = d.p + off;
  const int bc = d.ph.bc;
  double s2 = 0.0;
  for (int c = blockIdx.x * CG_THREADS + threadIdx.x; c < g.ncell; c += gridDim.x * CG_THREADS) {
    const int cy = c / g.nx, cx = c - cy * g.nx;
    if (cx < g.wx0 || cx > g.wx1) continue;
    const double pc = p[c];
    const double ap = -phi_at(p, g, bc, l, cx, cy - 1) - phi_at(p, g, bc, l, cx - 1, cy) + f4 * pc
                      - phi_at(p, g, bc, l, cx + 1, cy) - phi_at(p, g, bc, l, cx, cy + 1);
    d.ap[off + c] = ap;
    s2 = s2 + pc * ap;
  }
  s2 = block_sum(s2, sh);
  if (threadIdx.x == 0) {
    d.partials[((size_t)l * d.nred + blockIdx.x) * 2 + 0] = 0.0;
    d.partials[((size_t)l * d.nred + blockIdx.x) * 2 + 1] = s2;
  }
}

__global__ void __launch_bounds__(CG_THREADS) k_cg_ap_fin(Dev2D d) {
  __shared__ double sh[CG_THREADS];
  const int l = blockIdx.x;
  if (!d.cg[l].active) return;
  double dummy, s2;
  final_sums(d, l, sh, &dummy, &s2);
  if (threadIdx.x == 0) {
    CGState& st = d.cg[l];
    st.sum2_g = s2;
    st.av = st.sumr_g / s2;  // sumr_g: r.r of the current r (initial sum or the last sum1)
  }
}

// phi += av p ; r -= av ap ; partial of r.r
__global__ void __launch_bounds__(CG_THREADS) k_cg_update(Dev2D d) {
  __shared__ double sh[CG_THREADS];
  const Grid2D g = d.g;
  const int l = blockIdx.y;
  if (!d.cg[l].active) return;
  const size_t off = (size_t)l * g.ncell;
  const double av = d.cg[l].av;
  double s1 = 0.0;
  for (int c = blockIdx.x * CG_THREADS + threadIdx.x; c < g.ncell; c += gridDim.x * CG_THREADS) {
    const int cx = c % g.nx;
    if (cx < g.wx0 || cx > g.wx1) continue;
    d.phi[off + c] = d.phi[off + c] + av * d.p[off + c];
    const double r = d.r[off + c] - av * d.ap[off + c];
    d.r[off + c] = r;
    s1 = s1 + r * r;
  }
  s1 = block_sum(s1, sh);
  if (threadIdx.x == 0) {
    d.partials[((size_t)l * d.nred + blockIdx.x) * 2 + 0] = s1;
    d.partials[((size_t)l * d.nred + blockIdx.x) * 2 + 1] = 0.0;
  }
}

__global__ void __launch_bounds__(CG_THREADS) k_cg_update_fin(Dev2D d) {
  __shared__ double sh[CG_THREADS];
  const int l = blockIdx.x;
  if (!d.cg[l].active) return;
  double s1, dummy;
  final_sums(d, l, sh, &s1, &dummy);
  if (threadIdx.x == 0) {
    CGState& st = d.cg[l];
    st.sum_g = sqrt(st.sumr_g);
    st.ite = st.ite + 1;
    st.sum1_g = s1;
    st.bv = s1 / st.sumr_g;
    st.sumr_g = s1;  // r.r of the updated r: the next iteration's sumr
    bool cont = st.fixed >= 0 ? (st.ite < st.fixed) : (st.sum_g > st.eps);
    if (st.fixed < 0 && st.ite >= d.ite_max) {  // reference: write + stop (field.f90:427-430)
      atomicOr(d.err, EB_CG);
      cont = false;
    }
    // the active flag is cleared only after k_cg_p has consumed bv for a continuing component
    st.active = cont ? 1 : 2;
  }
}

// p = r + bv p, for components that continue; finishing components drop to inactive
__global__ void __launch_bounds__(CG_THREADS) k_cg_p(Dev2D d) {
  const Grid2D g = d.g;
  const int l = blockIdx.y;
  const int act = d.cg[l].active;
  if (act != 1) return;
  const size_t off = (size_t)l * g.ncell;
  const double bv = d.cg[l].bv;
  for (int c = blockIdx.x * CG_THREADS + threadIdx.x; c < g.ncell; c += gridDim.x * CG_THREADS) {
    const int cx = c % g.nx;
    if (cx < g.wx0 || cx > g.wx1) continue;
    d.p[off + c] = d.r[off + c] + bv * d.p[off + c];
  }
}

__global__ void k_cg_settle(Dev2D d) {
  if (threadIdx.x < 3 && d.cg[threadIdx.x].active == 2) d.cg[threadIdx.x].active = 0;
}

void cg_init2d(const Dev2D& d, cudaStream_t s) {
  k_cg_init<<<dim3(d.nred, 3), CG_THREADS, 0, s>>>(d);
  k_cg_init_fin<<<3, CG_THREADS, 0, s>>>(d);
}
void cg_iter_ap2d(const Dev2D& d, cudaStream_t s) {
  k_cg_ap<<<dim3(d.nred, 3), CG_THREADS, 0, s>>>(d);
  k_cg_ap_fin<<<3, CG_THREADS, 0, s>>>(d);
}
void cg_iter_update2d(const Dev2D& d, cudaStream_t s) {
  k_cg_update<<<dim3(d.nred, 3), CG_THREADS, 0, s>>>(d);
  k_cg_update_fin<<<3, CG_THREADS, 0, s>>>(d);
}
void cg_iter_p2d(const Dev2D& d, cudaStream_t s) {
  k_cg_p<<<dim3(d.nred, 3), CG_THREADS, 0, s>>>(d);
  k_cg_settle<<<1, 32, 0, s>>>(d);
}

// db(l, interior) = phi  (field.f90:455-457)
__global__ void k_cg_store(Dev2D d) {
  const Grid2D g = d.g;
  const int l = blockIdx.y;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < g.ncell; c += gridDim.x * blockDim.x) {
    const int cy = c / g.nx, cx = c - cy * g.nx;
    if (cx < g.wx0 || cx > g.wx1) continue;
    d.df[(size_t)l * g.fplane + (size_t)(cy + 2) * g.fp + cx + 2] = d.phi[(size_t)l * g.ncell + c];
  }
}
void cg_store2d(const Dev2D& d, cudaStream_t s) { k_cg_store<<<dim3(d.nred, 3), CG_THREADS, 0, s>>>(d); }

// ---------------------------------------------------------------------------
// E increment  (2d/common/field.f90:153-171)
// ---------------------------------------------------------------------------
__global__ void k_efield2d(Dev2D d) {
  const Grid2D g = d.g;
  const int cx = blockIdx.x * blockDim.x + threadIdx.x, cy = blockIdx.y;
  if (cx < g.wx0 || cx > g.wx1) return;
  const size_t f = (size_t)(cy + 2) * g.fp + (cx + 2);
  const size_t P = g.fplane;
  const size_t E = f + 1, N = f + g.fp;
  const double f1 = d.ph.f1, gfac = d.ph.gfac, pi = d.ph.pi, delt = d.ph.delt;
  const double* uf = d.uf;
  const double* df = d.df;
  const double* uj = d.uj;
#define U(c, at) uf[(c) * P + (at)]
#define D(c, at) df[(c) * P + (at)]
#define J(c, at) uj[(c) * P + (at)]
  const double d4 = +f1 * (+gfac * (-D(2, f) + D(2, N)) + (-U(2, f) + U(2, N))) - 4. * pi * delt * J(0, f);
  const double d5 = -f1 * (+gfac * (-D(2, f) + D(2, E)) + (-U(2, f) + U(2, E))) - 4. * pi * delt * J(1, f);
  const double d6 = +f1 * (+gfac * (-D(1, f) + D(1, E) + D(0, f) - D(0, N)) + (-U(1, f) + U(1, E) + U(0, f) - U(0, N)))
                    - 4. * pi * delt * J(2, f);
#undef U
#undef D
#undef J
  d.df[3 * P + f] = d4;
  d.df[4 * P + f] = d5;
  d.df[5 * P + f] = d6;
}

void efield2d(const Dev2D& d, cudaStream_t s) {
  dim3 grid((d.g.nx + 127) / 128, d.g.ny);
  k_efield2d<<<grid, 128, 0, s>>>(d);
}

// ---------------------------------------------------------------------------
// energy_history sums (2d/proj/weibel/app.f90:502-534), deterministic reductions.
// red_out = [vene(1), vene(2), sum E^2, sum B^2]
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(CG_THREADS) k_energy_parts(Dev2D d) {
  __shared__ double sh[CG_THREADS];
  const Grid2D g = d.g;
  const int isp = blockIdx.y;
  const double c = d.ph.c, rr = d.ph.r[isp];
  double v = 0.0;
  for (int jj = 0; jj < g.ny; ++jj) {
    const int row = isp * g.ny + jj;
    const int n = d.np2[row];
    const size_t rb = (size_t)row * d.cap;
    for (int s = blockIdx.x * CG_THREADS + threadIdx.x; s < n; s += gridDim.x * CG_THREADS) {
      const double a = d.A.ux[rb + s], b = d.A.uy[rb + s], e = d.A.uz[rb + s];
      const double u2 = a * a + b * b + e * e;
      const double gam = sqrt(1 + u2 / (c * c));
      v = v + rr * (gam - 1);
    }
  }
  v = block_sum(v, sh);
  if (threadIdx.x == 0) d.partials[((size_t)isp * d.nred + blockIdx.x) * 2] = v;
}

__global__ void __launch_bounds__(CG_THREADS) k_energy_fields(Dev2D d) {
  __shared__ double sh[CG_THREADS];
  const Grid2D g = d.g;
  double be = 0.0, ee = 0.0;
  for (int c = blockIdx.x * CG_THREADS + threadIdx.x; c < g.ncell; c += gridDim.x * CG_THREADS) {
    const int cy = c / g.nx, cx = c - cy * g.nx;
    const size_t f = (size_t)(cy + 2) * g.fp + cx + 2;
    const size_t P = g.fplane;
    const double b1 = d.uf[f], b2 = d.uf[P + f], b3 = d.uf[2 * P + f];
    const double e1 = d.uf[3 * P + f], e2 = d.uf[4 * P + f], e3 = d.uf[5 * P + f];
    be = be + b1 * b1 + b2 * b2 + b3 * b3;
    ee = ee + e1 * e1 + e2 * e2 + e3 * e3;
  }
  be = block_sum(be, sh);
  ee = block_sum(ee, sh);
  if (threadIdx.x == 0) {
    d.partials[((size_t)2 * d.nred + blockIdx.x) * 2 + 0] = ee;
    d.partials[((size_t)2 * d.nred + blockIdx.x) * 2 + 1] = be;
  }
}

__global__ void __launch_bounds__(CG_THREADS) k_energy_fin(Dev2D d) {
  __shared__ double sh[CG_THREADS];
  double a, b;
  final_sums(d, 0, sh, &a, &b);
  if (threadIdx.x == 0) d.red_out[0] = a;
  final_sums(d, 1, sh, &a, &b);
  if (threadIdx.x == 0) d.red_out[1] = a;
  final_sums(d, 2, sh, &a, &b);
  if (threadIdx.x == 0) {
    d.red_out[2] = a;
    d.red_out[3] = b;
  }
}

// partial slots [l][k][2]: l = 0,1 species kinetic (slot 0); l = 2 fields
void energy2d(const Dev2D& d, cudaStream_t s) {
  cudaMemsetAsync(d.partials, 0, sizeof(double) * 2 * 3 * (size_t)d.nred, s);
  k_energy_parts<<<dim3(d.nred, d.ph.nsp), CG_THREADS, 0, s>>>(d);
  energy_fields_fin2d(d, s);
}
void energy_fields_fin2d(const Dev2D& d, cudaStream_t s) {
  k_energy_fields<<<d.nred, CG_THREADS, 0, s>>>(d);
  k_energy_fin<<<1, CG_THREADS, 0, s>>>(d);
}
