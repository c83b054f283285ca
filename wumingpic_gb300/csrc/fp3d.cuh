// Precision-dependent 3D kernels of the FP64 path, included inside namespace
// wpic::exact (-fmad=false: every operation rounded separately in the
// reference's order) and inside namespace wpic::fast (FMA contraction allowed).
//
// Requires: wpic_internal.h, common.cuh, and fp2d.cuh (block_sum, CG_THREADS) before.

__device__ __forceinline__ size_t f3(const Grid3D& g, int fi, int fj, int fk) {  // ghosted field index
  return (size_t)fi + (size_t)g.fp * ((size_t)fj + (size_t)(g.ny + 4) * (size_t)fk);
}

// ---------------------------------------------------------------------------
// particle__solv  (3d/common/particle.f90:52-233)
// One CTA per (tile of PUSH_TW cells of a row (j, k), species).  The cell-centred
// E/B values tmpf(1:6, i-1:i+1, j-1:j+1, k-1:k+1) are formed once per tile in
// shared memory (particle.f90:75-92); each particle then gathers 27 points per
// component in the reference's nesting order.
// ---------------------------------------------------------------------------
// MODE PUSH_MOM is mom_calc__accl (3d/common/mom_calc.f90:49-216): the same gather and
// rotation at half the time step (mom_calc__init, :36), positions copied, no move.
template <int MODE>
__global__ void __launch_bounds__(PUSH_THREADS) k_push3d(Dev3D d) {
  constexpr bool VAY = MODE == PUSH_VAY;
  const Grid3D g = d.g;
  // blockIdx.x = x tile + tiles per row * (row of the species), blockIdx.y = species
  const int ntx = (g.nx + PUSH_TW - 1) / PUSH_TW;
  const int c0 = (blockIdx.x % ntx) * PUSH_TW;
  const int rs = blockIdx.x / ntx;
  const int jj = rs % g.ny, kk = rs / g.ny, isp = blockIdx.y;
  if (c0 >= g.nx) return;
  const int nc = min(PUSH_TW, g.nx - c0);
  __shared__ double tmp[6][3][3][PUSH_TW + 2];  // [comp][k-1..k+1][j-1..j+1][i]
  __shared__ int scc[PUSH_TW + 1];
  const int row = (isp * g.nz + kk) * g.ny + jj;
  for (int idx = threadIdx.x; idx < 9 * (nc + 2); idx += blockDim.x) {
    const int rk = idx / (3 * (nc + 2)), rem = idx - rk * 3 * (nc + 2);
    const int rj = rem / (nc + 2), ci = rem - rj * (nc + 2);
    // field index of cell (c0+ci-1, jj+rj-1, kk+rk-1)
    const int fi = c0 + ci + 1, fj = jj + rj + 1, fk = kk + rk + 1;
    const double* U = d.uf;
#define UF(c, di, dj, dk) U[(size_t)(c) * g.fvol + f3(g, fi + (di), fj + (dj), fk + (dk))]
    tmp[0][rk][rj][ci] = 2.5e-1 * (+UF(0, 0, 0, 0) + UF(0, 0, 1, 0) + UF(0, 0, 0, 1) + UF(0, 0, 1, 1));
    tmp[1][rk][rj][ci] = 2.5e-1 * (+UF(1, 0, 0, 0) + UF(1, 1, 0, 0) + UF(1, 0, 0, 1) + UF(1, 1, 0, 1));
    tmp[2][rk][rj][ci] = 2.5e-1 * (+UF(2, 0, 0, 0) + UF(2, 1, 0, 0) + UF(2, 0, 1, 0) + UF(2, 1, 1, 0));
    tmp[3][rk][rj][ci] = 5e-1 * (+UF(3, 0, 0, 0) + UF(3, 1, 0, 0));
    tmp[4][rk][rj][ci] = 5e-1 * (+UF(4, 0, 0, 0) + UF(4, 0, 1, 0));
    tmp[5][rk][rj][ci] = 5e-1 * (+UF(5, 0, 0, 0) + UF(5, 0, 0, 1));
#undef UF
  }
  for (int idx = threadIdx.x; idx <= nc; idx += blockDim.x) scc[idx] = d.cc[(size_t)row * (g.nx + 1) + c0 + idx];
  __syncthreads();

  const double dxi = d.ph.p_d_delx, delt = MODE == PUSH_MOM ? d.ph.delt * 5e-1 : d.ph.delt, c = d.ph.c;
  const double fac1 = d.ph.q[isp] / d.ph.r[isp] * 5e-1 * delt;
  const double txxx = fac1 * fac1;
  const double fac2 = d.ph.q[isp] * delt / d.ph.r[isp];
#if !WPIC_REF_ORDER
  const double ic2 = 1.0 / (c * c);
#endif
  const int jabs = g.nygs + jj, kabs = g.nzgs + kk;
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
    const double x = d.A.x[k], y = d.A.y[k], z = d.A.z[k];
    double dh = x * dxi - 5e-1 - (double)iabs;
    const double shxm = 5e-1 * (5e-1 - dh) * (5e-1 - dh), shx = 7.5e-1 - dh * dh, shxp = 5e-1 * (5e-1 + dh) * (5e-1 + dh);
    dh = y * dxi - 5e-1 - (double)jabs;
    const double shym = 5e-1 * (5e-1 - dh) * (5e-1 - dh), shy = 7.5e-1 - dh * dh, shyp = 5e-1 * (5e-1 + dh) * (5e-1 + dh);
    dh = z * dxi - 5e-1 - (double)kabs;
    const double shzm = 5e-1 * (5e-1 - dh) * (5e-1 - dh), shz = 7.5e-1 - dh * dh, shzp = 5e-1 * (5e-1 + dh) * (5e-1 + dh);
    double f[6];
#if WPIC_REF_ORDER
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      double pl[3];
#pragma unroll
      for (int rk = 0; rk < 3; ++rk) {
        const double r0 = +tmp[m][rk][0][lo] * shxm + tmp[m][rk][0][lo + 1] * shx + tmp[m][rk][0][lo + 2] * shxp;
        const double r1 = +tmp[m][rk][1][lo] * shxm + tmp[m][rk][1][lo + 1] * shx + tmp[m][rk][1][lo + 2] * shxp;
        const double r2 = +tmp[m][rk][2][lo] * shxm + tmp[m][rk][2][lo + 1] * shx + tmp[m][rk][2][lo + 2] * shxp;
        pl[rk] = +r0 * shym + r1 * shy + r2 * shyp;
      }
      f[m] = +pl[0] * shzm + pl[1] * shz + pl[2] * shzp;
    }
#else
    // FMA build: the 27 node weights once, then 27 fused multiply-adds per component (198 FP64
    // instructions for the gather instead of about 234; the FP64 pipe is the bound)
    {
      const double wx[3] = {shxm, shx, shxp}, wy[3] = {shym, shy, shyp}, wz[3] = {shzm, shz, shzp};
      double w[27];
#pragma unroll
      for (int rk = 0; rk < 3; ++rk)
#pragma unroll
        for (int rj = 0; rj < 3; ++rj) {
          const double wzy = wz[rk] * wy[rj];
#pragma unroll
          for (int ci = 0; ci < 3; ++ci) w[(rk * 3 + rj) * 3 + ci] = wzy * wx[ci];
        }
#pragma unroll
      for (int m = 0; m < 6; ++m) {
        double v = tmp[m][0][0][lo] * w[0];
#pragma unroll
        for (int q = 1; q < 27; ++q) v = fma(tmp[m][q / 9][(q / 3) % 3][lo + q % 3], w[q], v);
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
      d.B.z[k] = z + gv[2] * delt * ig;
      d.B.id[k] = d.A.id[k];
      continue;
    }
    double uvm1 = d.A.ux[k] + fac1 * epx;
    double uvm2 = d.A.uy[k] + fac1 * epy;
    double uvm3 = d.A.uz[k] + fac1 * epz;
#if WPIC_REF_ORDER
    double gam = sqrt(c * c + uvm1 * uvm1 + uvm2 * uvm2 + uvm3 * uvm3);
    const double igam = 1e0 / gam;
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
    const double g4 = uvm1 + fac1 * epx;
    const double g5 = uvm2 + fac1 * epy;
    const double g6 = uvm3 + fac1 * epz;
    if (MODE == PUSH_MOM) {
      d.B.x[k] = x;
      d.B.y[k] = y;
      d.B.z[k] = z;
      d.B.ux[k] = g4;
      d.B.uy[k] = g5;
      d.B.uz[k] = g6;
      continue;
    }
#if WPIC_REF_ORDER
    gam = 1e0 / sqrt(1e0 + (+g4 * g4 + g5 * g5 + g6 * g6) / (c * c));
#else
    gam = rsqrt(1e0 + (g4 * g4 + g5 * g5 + g6 * g6) * ic2);
#endif
    d.B.ux[k] = g4;
    d.B.uy[k] = g5;
    d.B.uz[k] = g6;
    d.B.x[k] = x + g4 * delt * gam;
    d.B.y[k] = y + g5 * delt * gam;
    d.B.z[k] = z + g6 * delt * gam;
    d.B.id[k] = d.A.id[k];
  }
}

void push3d(const Dev3D& d, cudaStream_t s) {
  dim3 grid(((d.g.nx + PUSH_TW - 1) / PUSH_TW) * d.g.ny * d.g.nz, d.ph.nsp);
  k_push3d<PUSH_BORIS><<<grid, PUSH_THREADS, 0, s>>>(d);
}

void push_vay3d(const Dev3D& d, cudaStream_t s) {
  dim3 grid(((d.g.nx + PUSH_TW - 1) / PUSH_TW) * d.g.ny * d.g.nz, d.ph.nsp);
  k_push3d<PUSH_VAY><<<grid, PUSH_THREADS, 0, s>>>(d);
}

void mom_accl3d(const Dev3D& d, cudaStream_t s) {
  dim3 grid(((d.g.nx + PUSH_TW - 1) / PUSH_TW) * d.g.ny * d.g.nz, d.ph.nsp);
  k_push3d<PUSH_MOM><<<grid, PUSH_THREADS, 0, s>>>(d);
}

// ---------------------------------------------------------------------------
// mom_calc__nvt  (3d/common/mom_calc.f90:219-332)
// One thread per node (I, J, K) of mom(7, nxgs-1:nxge+1, nys-1:nye+1, nzs-1:nze+1, nsp);
// it walks the particle rows (j, k) of K-1..K+1 and J-1..J+1 in the reference's loop
// order (k outer) and, within a row, cells I-1..I+1 in storage order, so each node is the
// single-thread reference's sum.  Node index floor(x/dx - 0.5) and offset x - 0.5 - ih as
// the 3D reference writes them; bucket-sorted particles required, as in 2D.
// ---------------------------------------------------------------------------
constexpr int MOM3_TX = 128;

__global__ void __launch_bounds__(MOM3_TX) k_mom_nvt3d(Dev3D d, Parts3D P, double* mom) {
  const Grid3D g = d.g;
  const int nxm = g.nx + 2, nym = g.ny + 2, nzm = g.nz + 2;
  const int nbx = (nxm + MOM3_TX - 1) / MOM3_TX;
  const int in = (blockIdx.x % nbx) * MOM3_TX + threadIdx.x, jn = blockIdx.x / nbx;
  const int kn = blockIdx.y, isp = blockIdx.z;
  if (in >= nxm) return;
  const int I = g.nxgs - 1 + in, J = g.nygs - 1 + jn, K = g.nzgs - 1 + kn;
  const double d_delx = d.ph.d_delx, c = d.ph.c;
  double acc[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  bool bad = false;
  const int c_lo = max(in - 2, 0), c_hi = min(in, g.nx - 1);  // cells I-1..I+1
  if (c_lo <= c_hi) {
    for (int dk = -1; dk <= 1; ++dk) {
      const int kk = kn - 1 + dk;
      if (kk < 0 || kk >= g.nz) continue;
      for (int dj = -1; dj <= 1; ++dj) {
        const int jj = jn - 1 + dj;
        if (jj < 0 || jj >= g.ny) continue;
        const int row = (isp * g.nz + kk) * g.ny + jj;
        const int* ccr = d.cc + (size_t)row * (g.nx + 1);
        const int s0 = ccr[c_lo], s1 = ccr[c_hi + 1];
        const bool own_row = dj == 0 && dk == 0 && in >= 1 && in <= g.nx;
        const int own0 = own_row ? ccr[in - 1] : 0, own1 = own_row ? ccr[in] : 0;
        const size_t rbase = (size_t)row * d.cap;
        for (int s = s0; s < s1; ++s) {
          const size_t k = rbase + s;
          const double x = P.x[k], y = P.y[k], z = P.z[k];
          const int ih = (int)floor(x * d_delx - 5e-1);
          const int jh = (int)floor(y * d_delx - 5e-1);
          const int kh = (int)floor(z * d_delx - 5e-1);
          if (s >= own0 && s < own1 &&
              (ih < I - 1 || ih > I || jh < J - 1 || jh > J || kh < K - 1 || kh > K))
            bad = true;
          const int a = I - ih, b = J - jh, e = K - kh;
          if (a < 0 || a > 1 || b < 0 || b > 1 || e < 0 || e > 1) continue;
          const double dx = x - 5e-1 - ih, dxm = 1e0 - dx;
          const double dy = y - 5e-1 - jh, dym = 1e0 - dy;
          const double dz = z - 5e-1 - kh, dzm = 1e0 - dz;
          const double wx = a ? dx : dxm, wy = b ? dy : dym, wz = e ? dz : dzm;
          const double u1 = P.ux[k], u2 = P.uy[k], u3 = P.uz[k];
          const double gam = 1e0 / sqrt(1e0 + (+u1 * u1 + u2 * u2 + u3 * u3) / (c * c));
          acc[0] = acc[0] + wx * wy * wz;
          acc[1] = acc[1] + u1 * gam * wx * wy * wz;
          acc[2] = acc[2] + u2 * gam * wx * wy * wz;
          acc[3] = acc[3] + u3 * gam * wx * wy * wz;
          acc[4] = acc[4] + u1 * u1 * gam * wx * wy * wz;
          acc[5] = acc[5] + u2 * u2 * gam * wx * wy * wz;
          acc[6] = acc[6] + u3 * u3 * gam * wx * wy * wz;
        }
      }
    }
  }
  if (bad) atomicOr(d.err, EB_OUT_OF_RANGE);
  double* o = mom + 7 * ((size_t)in + (size_t)nxm * ((size_t)jn + (size_t)nym * ((size_t)kn + (size_t)nzm * isp)));
#pragma unroll
  for (int l = 0; l < 7; ++l) o[l] = acc[l];
}

#if !WPIC_REF_ORDER
// The FMA build, as in 2D: one thread per cell sums its particles' seven moments into the
// cell's 3 x 3 x 3 node tile (189 values, the first of the deposit's 375 per cell), then a
// per-node gather of the 27 tiles that touch each node; within 1e-12 of the reference order.
constexpr int MOMC3_T = 32;

__global__ void __launch_bounds__(MOMC3_T) k_mom_cell3d(Dev3D d, Parts3D P, int isp) {
  extern __shared__ double macc3[];  // [189][MOMC3_T]: moment l of tile node (ta, tb, tc) at l + 7 (ta + 3 (tb + 3 tc))
  const Grid3D g = d.g;
  const int cx = blockIdx.x * MOMC3_T + threadIdx.x, jj = blockIdx.y, kk = blockIdx.z;
  if (cx >= g.nx) return;
  double* a = macc3 + threadIdx.x;
  for (int e = 0; e < 189; ++e) a[e * MOMC3_T] = 0.0;
  const double d_delx = d.ph.d_delx, c = d.ph.c, ic2 = 1.0 / (c * c);
  const int row = (isp * g.nz + kk) * g.ny + jj;
  const int* ccr = d.cc + (size_t)row * (g.nx + 1);
  const int i0 = g.nxgs - 1 + cx, j0 = g.nygs - 1 + jj, k0 = g.nzgs - 1 + kk;
  const size_t rbase = (size_t)row * d.cap;
  bool bad = false;
  for (int sl = ccr[cx]; sl < ccr[cx + 1]; ++sl) {
    const size_t k = rbase + sl;
    const double x = P.x[k], y = P.y[k], z = P.z[k];
    const int ih = (int)floor(x * d_delx - 5e-1), jh = (int)floor(y * d_delx - 5e-1), kh = (int)floor(z * d_delx - 5e-1);
    const int ta = ih - i0, tb = jh - j0, tc = kh - k0;
    if (ta < 0 || ta > 1 || tb < 0 || tb > 1 || tc < 0 || tc > 1) {
      bad = true;
      continue;
    }
    const double dx = x - 5e-1 - ih, dy = y - 5e-1 - jh, dz = z - 5e-1 - kh;  // as the 3D reference writes them
    const double u1 = P.ux[k], u2 = P.uy[k], u3 = P.uz[k];
    const double gam = 1e0 / sqrt(1e0 + (u1 * u1 + u2 * u2 + u3 * u3) * ic2);
    const double pre[7] = {1.0, u1 * gam, u2 * gam, u3 * gam, u1 * u1 * gam, u2 * u2 * gam, u3 * u3 * gam};
    const double wx[2] = {1e0 - dx, dx}, wy[2] = {1e0 - dy, dy}, wz[2] = {1e0 - dz, dz};
#pragma unroll
    for (int e = 0; e < 2; ++e)
#pragma unroll
      for (int b = 0; b < 2; ++b) {
        const double wyz = wy[b] * wz[e];
#pragma unroll
        for (int aa = 0; aa < 2; ++aa) {
          const double w = wx[aa] * wyz;
          double* t = a + 7 * ((ta + aa) + 3 * ((tb + b) + 3 * (tc + e))) * MOMC3_T;
#pragma unroll
          for (int l = 0; l < 7; ++l) t[l * MOMC3_T] = fma(pre[l], w, t[l * MOMC3_T]);
        }
      }
  }
  if (bad) atomicOr(d.err, EB_OUT_OF_RANGE);
  double* out = d.cellJ + ((size_t)kk * g.ny * g.nx + (size_t)jj * g.nx + cx) * 189;
  for (int e = 0; e < 189; ++e) out[e] = a[e * MOMC3_T];
}

__global__ void k_mom_gather3d(Dev3D d, double* mom, int isp) {
  const Grid3D g = d.g;
  const int nxm = g.nx + 2, nym = g.ny + 2, nzm = g.nz + 2;
  const int in = blockIdx.x * blockDim.x + threadIdx.x, jn = blockIdx.y, kn = blockIdx.z;
  if (in >= nxm) return;
  double acc[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int tc = 0; tc < 3; ++tc) {
    const int kk = kn - tc;
    if (kk < 0 || kk >= g.nz) continue;
    for (int tb = 0; tb < 3; ++tb) {
      const int jj = jn - tb;
      if (jj < 0 || jj >= g.ny) continue;
      for (int ta = 0; ta < 3; ++ta) {
        const int cx = in - ta;
        if (cx < 0 || cx >= g.nx) continue;
        const double* t = d.cellJ + ((size_t)kk * g.ny * g.nx + (size_t)jj * g.nx + cx) * 189 + 7 * (ta + 3 * (tb + 3 * tc));
#pragma unroll
        for (int l = 0; l < 7; ++l) acc[l] += t[l];
      }
    }
  }
  double* o = mom + 7 * ((size_t)in + (size_t)nxm * ((size_t)jn + (size_t)nym * ((size_t)kn + (size_t)nzm * isp)));
#pragma unroll
  for (int l = 0; l < 7; ++l) o[l] = acc[l];
}
#endif

void mom_nvt3d(const Dev3D& d, const Parts3D& P, double* mom, cudaStream_t s) {
#if WPIC_REF_ORDER
  const int nbx = (d.g.nx + 2 + MOM3_TX - 1) / MOM3_TX;
  dim3 grid(nbx * (d.g.ny + 2), d.g.nz + 2, d.ph.nsp);
  k_mom_nvt3d<<<grid, MOM3_TX, 0, s>>>(d, P, mom);
#else
  for (int isp = 0; isp < d.ph.nsp; ++isp) {
    k_mom_cell3d<<<dim3((d.g.nx + MOMC3_T - 1) / MOMC3_T, d.g.ny, d.g.nz), MOMC3_T, 189 * MOMC3_T * sizeof(double),
                   s>>>(d, P, isp);
    k_mom_gather3d<<<dim3((d.g.nx + 2 + 127) / 128, d.g.ny + 2, d.g.nz + 2), 128, 0, s>>>(d, mom, isp);
  }
#endif
}

// ---------------------------------------------------------------------------
// ele_cur  (3d/common/field.f90:211-406)
// One thread per cell walks the cell's particles of both species in bucket order
// and accumulates the cell's 5x5x5 stencils pjx, pjy, pjz (shared memory, one
// column per thread) exactly as the reference; the 375 values go to cellJ and
// k_jgather3d adds them into uj in the reference's (k, j, i) cell order, the
// single-thread OpenMP reduction order.  Storage of one stencil:
// pj[comp][kp][jp][a], a = the offset along the current's own axis (the
// reference's first index), jp/kp its two loop indices.
// ---------------------------------------------------------------------------
constexpr int DEP3_THREADS = 32;
constexpr int DEP3_VALS = 375;

__global__ void __launch_bounds__(DEP3_THREADS) k_deposit3d(Dev3D d) {
  extern __shared__ double acc3[];  // [375][DEP3_THREADS]
  const Grid3D g = d.g;
  const int cx = blockIdx.x * DEP3_THREADS + threadIdx.x;
  const int jj = blockIdx.y, kk = blockIdx.z;
  if (cx >= g.nx) return;
  double* a = acc3 + threadIdx.x;
  for (int e = 0; e < DEP3_VALS; ++e) a[e * DEP3_THREADS] = 0.0;
  const double d_delx = d.ph.d_delx, d_delt = d.ph.d_delt, delx = d.ph.delx;
  const double fac = 1.0 / 3.0;
  const int cell[3] = {g.nxgs + cx, g.nygs + jj, g.nzgs + kk};
  for (int isp = 0; isp < d.ph.nsp; ++isp) {
    const int row = (isp * g.nz + kk) * g.ny + jj;
    const int* ccr = d.cc + (size_t)row * (g.nx + 1);
    const int s0i = ccr[cx], s1i = ccr[cx + 1];
    const double qdxdt = d.ph.q[isp] * delx * d_delt;
    const size_t rbase = (size_t)row * d.cap;
    for (int s = s0i; s < s1i; ++s) {
      const size_t k = rbase + s;
      double s0[3][5], ds[3][5];
      const double po[3] = {d.A.x[k], d.A.y[k], d.A.z[k]};
      const double pn[3] = {d.B.x[k], d.B.y[k], d.B.z[k]};
#pragma unroll
      for (int dim = 0; dim < 3; ++dim) {
        const double dh = po[dim] * d_delx - 5e-1 - (double)cell[dim];
        s0[dim][0] = 0.0;
        s0[dim][1] = 5e-1 * (5e-1 - dh) * (5e-1 - dh);
        s0[dim][2] = 7.5e-1 - dh * dh;
        s0[dim][3] = 5e-1 * (5e-1 + dh) * (5e-1 + dh);
        s0[dim][4] = 0.0;
      }
#pragma unroll
      for (int dim = 0; dim < 3; ++dim) {
        const int i2 = (int)(pn[dim] * d_delx);
        const double dh1 = pn[dim] * d_delx - 5e-1 - (double)i2;
        const int inc = i2 - cell[dim];
        if (inc < -1 || inc > 1) atomicOr(d.err, EB_MOVED_TOO_FAR);
        const double s1_1 = 5e-1 * (5e-1 - dh1) * (5e-1 - dh1);
        const double s1_2 = 7.5e-1 - dh1 * dh1;
        const double s1_3 = 5e-1 * (5e-1 + dh1) * (5e-1 + dh1);
        const int ainc = inc < 0 ? -inc : inc;
        const double smo_1 = (double)(-(inc - ainc)) * 5e-1;
        const double smo_2 = (double)(-ainc + 1);
        const double smo_3 = (double)(inc + ainc) * 5e-1;
        ds[dim][0] = s1_1 * smo_1 - s0[dim][0];
        ds[dim][1] = s1_1 * smo_2 + s1_2 * smo_1 - s0[dim][1];
        ds[dim][2] = s1_2 * smo_2 + s1_3 * smo_1 + s1_1 * smo_3 - s0[dim][2];
        ds[dim][3] = s1_3 * smo_2 + s1_2 * smo_3 - s0[dim][3];
        ds[dim][4] = s1_3 * smo_3 - s0[dim][4];
      }
#if !WPIC_REF_ORDER
      // The same sums in factored form: per axis the weights q dx/dt (s0 + ds/2) and
      // q dx/dt (s0/2 + ds/3) and the prefix sums of ds, once per particle; every stencil entry is
      // then one fused multiply-add into its accumulator (about 500 instead of 1050 FP64
      // instructions per particle; the FP64 pipe is the bound).
      {
        double wa[3][5], wb[3][5], pre[3][4];
#pragma unroll
        for (int dim = 0; dim < 3; ++dim) {
#pragma unroll
          for (int e = 0; e < 5; ++e) {
            wa[dim][e] = (s0[dim][e] + 5e-1 * ds[dim][e]) * qdxdt;
            wb[dim][e] = (5e-1 * s0[dim][e] + fac * ds[dim][e]) * qdxdt;
          }
          pre[dim][0] = ds[dim][0];
#pragma unroll
          for (int q = 1; q < 4; ++q) pre[dim][q] = pre[dim][q - 1] + ds[dim][q];
        }
#pragma unroll 1
        for (int kp = 0; kp < 5; ++kp) {
#pragma unroll
          for (int jp = 0; jp < 5; ++jp) {
#pragma unroll
            for (int comp = 0; comp < 3; ++comp) {
              const int t1 = comp == 0 ? 1 : 0;
              const int t2 = comp == 2 ? 1 : 2;
              const double dstmp = fma(wa[t1][jp], s0[t2][kp], wb[t1][jp] * ds[t2][kp]);
              double* e = a + (size_t)(((comp * 5 + kp) * 5 + jp) * 5) * DEP3_THREADS;
#pragma unroll
              for (int q = 0; q < 4; ++q) e[(q + 1) * DEP3_THREADS] = fma(-pre[comp][q], dstmp, e[(q + 1) * DEP3_THREADS]);
            }
          }
        }
      }
#else
      // (field.f90:331-381): for every (jp, kp), the prefix along the component's own axis
#pragma unroll 1
      for (int kp = 0; kp < 5; ++kp) {
#pragma unroll
        for (int jp = 0; jp < 5; ++jp) {
#pragma unroll
          for (int comp = 0; comp < 3; ++comp) {
            // transverse axes (t1 indexed by jp, t2 by kp) and the own axis of each component
            const int t1 = comp == 0 ? 1 : 0;
            const int t2 = comp == 2 ? 1 : 2;
            const double dstmp = ((s0[t1][jp] + 5e-1 * ds[t1][jp]) * s0[t2][kp] +
                                  (5e-1 * s0[t1][jp] + fac * ds[t1][jp]) * ds[t2][kp]) * qdxdt;
            double* e = a + (size_t)(((comp * 5 + kp) * 5 + jp) * 5) * DEP3_THREADS;
            double pjtmp = -ds[comp][0] * dstmp;
            e[1 * DEP3_THREADS] = e[1 * DEP3_THREADS] + pjtmp;
            pjtmp = pjtmp - ds[comp][1] * dstmp;
            e[2 * DEP3_THREADS] = e[2 * DEP3_THREADS] + pjtmp;
            pjtmp = pjtmp - ds[comp][2] * dstmp;
            e[3 * DEP3_THREADS] = e[3 * DEP3_THREADS] + pjtmp;
            pjtmp = pjtmp - ds[comp][3] * dstmp;
            e[4 * DEP3_THREADS] = e[4 * DEP3_THREADS] + pjtmp;
          }
        }
      }
#endif
    }
  }
  double* out = d.cellJ + ((size_t)kk * g.ny * g.nx + (size_t)jj * g.nx + cx) * DEP3_VALS;
  for (int e = 0; e < DEP3_VALS; ++e) out[e] = a[e * DEP3_THREADS];
}

// uj(comp, node) = sum over the cells (kc, jc, ic) ascending of the cell's stencil value at the node;
// the node offset (ox, oy, oz) = node - cell maps to the stencil entry
// comp 0: pjx(ox, oy, oz); comp 1: pjy(oy, ox, oz); comp 2: pjz(oz, ox, oy)   (field.f90:391-401)
__global__ void k_jgather3d(Dev3D d) {
  const Grid3D g = d.g;
  const size_t nnode = g.fvol;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < 3 * nnode; t += (size_t)gridDim.x * blockDim.x) {
    const int comp = (int)(t / nnode);
    const size_t node = t - (size_t)comp * nnode;
    const int fi = (int)(node % g.fp);
    const int fj = (int)((node / g.fp) % (g.ny + 4));
    const int fk = (int)(node / g.fplane);
    // node in interior-cell coordinates: cell index = field index - 2
    const int ni = fi - 2, nj = fj - 2, nk = fk - 2;
    double sum = 0.0;
    for (int kc = nk - 2; kc <= nk + 2; ++kc) {
      if (kc < 0 || kc >= g.nz) continue;
      for (int jc = nj - 2; jc <= nj + 2; ++jc) {
        if (jc < 0 || jc >= g.ny) continue;
        for (int ic = ni - 2; ic <= ni + 2; ++ic) {
          if (ic < 0 || ic >= g.nx) continue;
          const int ox = ni - ic + 2, oy = nj - jc + 2, oz = nk - kc + 2;  // 0..4
          int a, jp, kp;
          if (comp == 0) { a = ox; jp = oy; kp = oz; }
          else if (comp == 1) { a = oy; jp = ox; kp = oz; }
          else { a = oz; jp = ox; kp = oy; }
          const size_t cid = ((size_t)kc * g.ny + jc) * g.nx + ic;
          sum = sum + d.cellJ[cid * DEP3_VALS + ((comp * 5 + kp) * 5 + jp) * 5 + a];
        }
      }
    }
    d.uj[t] = sum;
  }
}

void deposit3d(const Dev3D& d, cudaStream_t s) {
  dim3 grid((d.g.nx + DEP3_THREADS - 1) / DEP3_THREADS, d.g.ny, d.g.nz);
  const size_t shm = sizeof(double) * DEP3_VALS * DEP3_THREADS;
  cudaFuncSetAttribute(k_deposit3d, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  k_deposit3d<<<grid, DEP3_THREADS, shm, s>>>(d);
  k_jgather3d<<<8 * 152, 256, 0, s>>>(d);
}

// ---------------------------------------------------------------------------
// RHS gkl of the implicit B solve  (3d/common/field.f90:127-160)
// ---------------------------------------------------------------------------
__global__ void k_gkl3d(Dev3D d) {
  const Grid3D g = d.g;
  const size_t ncell = g.ncell;
  for (size_t cid = (size_t)blockIdx.x * blockDim.x + threadIdx.x; cid < ncell; cid += (size_t)gridDim.x * blockDim.x) {
    const int cx = (int)(cid % g.nx), cy = (int)((cid / g.nx) % g.ny), cz = (int)(cid / ((size_t)g.nx * g.ny));
    if (cx < g.wx0 || cx > g.wx1) continue;  // the active window nxs..nxe
    const size_t f = f3(g, cx + 2, cy + 2, cz + 2);
    const size_t V = g.fvol;
    const size_t W = f - 1, E = f + 1, S = f - g.fp, N = f + g.fp, B = f - g.fplane, T = f + g.fplane;
    const double* uf = d.uf;
    const double* uj = d.uj;
    const double f1 = d.ph.f1, f2 = d.ph.f2, f3c = d.ph.f3;
#define U(c, at) uf[(c) * V + (at)]
#define J(c, at) uj[(c) * V + (at)]
    const double g1 = +f2 * (+U(0, B) + U(0, S) + U(0, W) - 6e0 * U(0, f) + U(0, E) + U(0, N) + U(0, T) +
                             f3c * (-J(2, S) + J(2, f) + J(1, B) - J(1, f))) -
                      f1 * (-U(5, S) + U(5, f) + U(4, B) - U(4, f));
    const double g2 = +f2 * (+U(1, B) + U(1, S) + U(1, W) - 6e0 * U(1, f) + U(1, E) + U(1, N) + U(1, T) +
                             f3c * (-J(0, B) + J(0, f) + J(2, W) - J(2, f))) -
                      f1 * (-U(3, B) + U(3, f) + U(5, W) - U(5, f));
    const double g3 = +f2 * (+U(2, B) + U(2, S) + U(2, W) - 6e0 * U(2, f) + U(2, E) + U(2, N) + U(2, T) +
                             f3c * (-J(1, W) + J(1, f) + J(0, S) - J(0, f))) -
                      f1 * (-U(4, W) + U(4, f) + U(3, S) - U(3, f));
#undef U
#undef J
    d.gkl[cid] = g1;
    d.gkl[ncell + cid] = g2;
    d.gkl[2 * ncell + cid] = g3;
  }
}

void gkl3d(const Dev3D& d, cudaStream_t s) { k_gkl3d<<<8 * 152, 256, 0, s>>>(d); }

// ---------------------------------------------------------------------------
// cgm  (3d/common/field.f90:409-560): the three components side by side, the 2D
// path's deterministic reductions and stopping rule, a 6-neighbour stencil with
// periodic ghosts (boundary_periodic__phi, 3d/common/boundary_periodic.f90:981-1099)
// applied by index arithmetic.
// ---------------------------------------------------------------------------
// the value of component l at cell (x, y, z) one step outside the interior: periodic in y and z;
// in x periodic, or at conducting walls (boundary_reconnection__phi,
// 3d/proj/reconnection/boundary_reconnection.f90:1093-1117) component 1 odd about nxs and nxe-1,
// components 2 and 3 even about nxs and nxe
// Ghosts are taken at the edges of the active window nxs..nxe (cells wx0..wx1); beyond a shock
// run's nxe the value is zero (boundary_shock__phi, 3d/proj/shock/boundary_shock.f90:1084-1107).
// x0 = -1 marks that zero.
__device__ __forceinline__ void phi3_src(const Grid3D& g, int bc, int l, int& x, int& y, int& z, bool& neg) {
  if (y < 0) y += g.ny; else if (y >= g.ny) y -= g.ny;
  if (z < 0) z += g.nz; else if (z >= g.nz) z -= g.nz;
  neg = false;
  if (x < g.wx0) {
    if (bc == BC_PERIODIC) x += g.nx;
    else if (l == 0) { x = g.wx0; neg = true; }
    else x = g.wx0 + 1;
  } else if (x > g.wx1) {
    if (bc == BC_PERIODIC) x -= g.nx;
    else if (bc == BC_SHOCK) x = -1;
    else if (l == 0) { x = g.wx1 - 2; neg = true; }
    else x = g.wx1 - 1;
  }
}
__device__ __forceinline__ double v3_at(const double* v, const Grid3D& g, int bc, int l, int x, int y, int z) {
  bool neg;
  phi3_src(g, bc, l, x, y, z, neg);
  if (x < 0) return 0.0;
  return flip_sign(v[((size_t)z * g.ny + y) * g.nx + x], neg);
}

__device__ __forceinline__ void final_sums3(const Dev3D& d, int l, double* sh, double* out0, double* out1) {
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

__global__ void __launch_bounds__(CG_THREADS) k_cg3_init(Dev3D d) {
  __shared__ double sh[CG_THREADS];
  const Grid3D g = d.g;
  const int l = blockIdx.y;
  const size_t off = (size_t)l * g.ncell;
  const double f4 = d.ph.f4, f5 = d.ph.f5;
  // phi = db(l) over the interior, viewed with periodic ghosts
  const double* db = d.df + (size_t)l * g.fvol;
  const int bc = d.ph.bc;
  auto ph = [&](int x, int y, int z) {
    bool neg;
    phi3_src(g, bc, l, x, y, z, neg);
    if (x < 0) return 0.0;
    return flip_sign(db[f3(g, x + 2, y + 2, z + 2)], neg);
  };
  double sb = 0.0, sr = 0.0;
  for (size_t c = (size_t)blockIdx.x * CG_THREADS + threadIdx.x; c < g.ncell; c += (size_t)gridDim.x * CG_THREADS) {
    const int cx = (int)(c % g.nx), cy = (int)((c / g.nx) % g.ny), cz = (int)(c / ((size_t)g.nx * g.ny));
    if (cx < g.wx0 || cx > g.wx1) continue;  // outside the active window: not part of the system
    const double pc = ph(cx, cy, cz);
    const double b = f5 * d.gkl[off + c];
    const double r = b + ph(cx, cy, cz - 1) + ph(cx, cy - 1, cz) + ph(cx - 1, cy, cz) - f4 * pc + ph(cx + 1, cy, cz) +
                     ph(cx, cy + 1, cz) + ph(cx, cy, cz + 1);
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

__global__ void __launch_bounds__(CG_THREADS) k_cg3_init_fin(Dev3D d) {
  __shared__ double sh[CG_THREADS];
  const int l = blockIdx.x;
  double sb, sr;
  final_sums3(d, l, sh, &sb, &sr);
  if (threadIdx.x == 0) {
    CGState& st = d.cg[l];
    st.sum_g = sb;
    st.eps = sqrt(sb) * 1e-6;
    st.sumr_g = sr;
    st.ite = 0;
    if (st.fixed >= 0) st.active = st.fixed > 0;
    else st.active = (sqrt(sr) > st.eps) && (st.sum_g > st.eps);
  }
}

// ap = (f4 - N) p ; partial of p.ap (r.r carried from the previous sum, as in the 2D path)
__global__ void __launch_bounds__(CG_THREADS) k_cg3_ap(Dev3D d) {
  __shared__ double sh[CG_THREADS];
  const Grid3D g = d.g;
  const int l = blockIdx.y;
  if (!d.cg[l].active) return;
  const size_t off = (size_t)l * g.ncell;
  const double f4 = d.ph.f4;
  const double* p = d.p + off;
  double s2 = 0.0;
  for (size_t c = (size_t)blockIdx.x * CG_THREADS + threadIdx.x; c < g.ncell; c += (size_t)gridDim.x * CG_THREADS) {
    const int cx = (int)(c % g.nx), cy = (int)((c / g.nx) % g.ny), cz = (int)(c / ((size_t)g.nx * g.ny));
    if (cx < g.wx0 || cx > g.wx1) continue;
    const double pc = p[c];
    const int bc = d.ph.bc;
    const double ap = -v3_at(p, g, bc, l, cx, cy, cz - 1) - v3_at(p, g, bc, l, cx, cy - 1, cz) -
                      v3_at(p, g, bc, l, cx - 1, cy, cz) + f4 * pc - v3_at(p, g, bc, l, cx + 1, cy, cz) -
                      v3_at(p, g, bc, l, cx, cy + 1, cz) - v3_at(p, g, bc, l, cx, cy, cz + 1);
    d.ap[off + c] = ap;
    s2 = s2 + pc * ap;
  }
  s2 = block_sum(s2, sh);
  if (threadIdx.x == 0) {
    d.partials[((size_t)l * d.nred + blockIdx.x) * 2 + 0] = 0.0;
    d.partials[((size_t)l * d.nred + blockIdx.x) * 2 + 1] = s2;
  }
}

__global__ void __launch_bounds__(CG_THREADS) k_cg3_ap_fin(Dev3D d) {
  __shared__ double sh[CG_THREADS];
  const int l = blockIdx.x;
  if (!d.cg[l].active) return;
  double dummy, s2;
  final_sums3(d, l, sh, &dummy, &s2);
  if (threadIdx.x == 0) {
    CGState& st = d.cg[l];
    st.sum2_g = s2;
    st.av = st.sumr_g / s2;
  }
}

__global__ void __launch_bounds__(CG_THREADS) k_cg3_update(Dev3D d) {
  __shared__ double sh[CG_THREADS];
  const Grid3D g = d.g;
  const int l = blockIdx.y;
  if (!d.cg[l].active) return;
  const size_t off = (size_t)l * g.ncell;
  const double av = d.cg[l].av;
  double s1 = 0.0;
  for (size_t c = (size_t)blockIdx.x * CG_THREADS + threadIdx.x; c < g.ncell; c += (size_t)gridDim.x * CG_THREADS) {
    const int cx = (int)(c % g.nx);
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

__global__ void __launch_bounds__(CG_THREADS) k_cg3_update_fin(Dev3D d) {
  __shared__ double sh[CG_THREADS];
  const int l = blockIdx.x;
  if (!d.cg[l].active) return;
  double s1, dummy;
  final_sums3(d, l, sh, &s1, &dummy);
  if (threadIdx.x == 0) {
    CGState& st = d.cg[l];
    st.sum_g = sqrt(st.sumr_g);
    st.ite = st.ite + 1;
    st.sum1_g = s1;
    st.bv = s1 / st.sumr_g;
    st.sumr_g = s1;
    bool cont = st.fixed >= 0 ? (st.ite < st.fixed) : (st.sum_g > st.eps);
    if (st.fixed < 0 && st.ite >= d.ite_max) {  // reference: write + stop (field.f90:527-530)
      atomicOr(d.err, EB_CG);
      cont = false;
    }
    st.active = cont ? 1 : 2;
  }
}

__global__ void __launch_bounds__(CG_THREADS) k_cg3_p(Dev3D d) {
  const Grid3D g = d.g;
  const int l = blockIdx.y;
  if (d.cg[l].active != 1) return;
  const size_t off = (size_t)l * g.ncell;
  const double bv = d.cg[l].bv;
  for (size_t c = (size_t)blockIdx.x * CG_THREADS + threadIdx.x; c < g.ncell; c += (size_t)gridDim.x * CG_THREADS) {
    const int cx = (int)(c % g.nx);
    if (cx < g.wx0 || cx > g.wx1) continue;
    d.p[off + c] = d.r[off + c] + bv * d.p[off + c];
  }
}

__global__ void k_cg3_settle(Dev3D d) {
  if (threadIdx.x < 3 && d.cg[threadIdx.x].active == 2) d.cg[threadIdx.x].active = 0;
}

// db(l, interior) = phi  (field.f90:555-557)
__global__ void k_cg3_store(Dev3D d) {
  const Grid3D g = d.g;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < 3 * g.ncell; t += (size_t)gridDim.x * blockDim.x) {
    const int l = (int)(t / g.ncell);
    const size_t c = t - (size_t)l * g.ncell;
    const int cx = (int)(c % g.nx), cy = (int)((c / g.nx) % g.ny), cz = (int)(c / ((size_t)g.nx * g.ny));
    if (cx < g.wx0 || cx > g.wx1) continue;
    d.df[(size_t)l * g.fvol + f3(g, cx + 2, cy + 2, cz + 2)] = d.phi[t];
  }
}

void cg_init3d(const Dev3D& d, cudaStream_t s) {
  k_cg3_init<<<dim3(d.nred, 3), CG_THREADS, 0, s>>>(d);
  k_cg3_init_fin<<<3, CG_THREADS, 0, s>>>(d);
}
void cg_iter_ap3d(const Dev3D& d, cudaStream_t s) {
  k_cg3_ap<<<dim3(d.nred, 3), CG_THREADS, 0, s>>>(d);
  k_cg3_ap_fin<<<3, CG_THREADS, 0, s>>>(d);
}
void cg_iter_update3d(const Dev3D& d, cudaStream_t s) {
  k_cg3_update<<<dim3(d.nred, 3), CG_THREADS, 0, s>>>(d);
  k_cg3_update_fin<<<3, CG_THREADS, 0, s>>>(d);
}
void cg_iter_p3d(const Dev3D& d, cudaStream_t s) {
  k_cg3_p<<<dim3(d.nred, 3), CG_THREADS, 0, s>>>(d);
  k_cg3_settle<<<1, 32, 0, s>>>(d);
}
void cg_store3d(const Dev3D& d, cudaStream_t s) { k_cg3_store<<<8 * 152, 256, 0, s>>>(d); }

// ---------------------------------------------------------------------------
// E update  (3d/common/field.f90:166-192)
// ---------------------------------------------------------------------------
__global__ void k_efield3d(Dev3D d) {
  const Grid3D g = d.g;
  for (size_t cid = (size_t)blockIdx.x * blockDim.x + threadIdx.x; cid < g.ncell; cid += (size_t)gridDim.x * blockDim.x) {
    const int cx = (int)(cid % g.nx), cy = (int)((cid / g.nx) % g.ny), cz = (int)(cid / ((size_t)g.nx * g.ny));
    if (cx < g.wx0 || cx > g.wx1) continue;  // the active window nxs..nxe
    const size_t f = f3(g, cx + 2, cy + 2, cz + 2);
    const size_t V = g.fvol;
    const size_t E = f + 1, N = f + g.fp, T = f + g.fplane;
    const double* uf = d.uf;
    double* df = d.df;
    const double f1 = d.ph.f1, gfac = d.ph.gfac, pi = d.ph.pi, delt = d.ph.delt;
#define U(c, at) uf[(c) * V + (at)]
#define D(c, at) df[(c) * V + (at)]
    const double e4 = +f1 * (+gfac * (-D(2, f) + D(2, N) + D(1, f) - D(1, T)) + (-U(2, f) + U(2, N) + U(1, f) - U(1, T))) -
                      4e0 * pi * delt * d.uj[0 * V + f];
    const double e5 = +f1 * (+gfac * (-D(0, f) + D(0, T) + D(2, f) - D(2, E)) + (-U(0, f) + U(0, T) + U(2, f) - U(2, E))) -
                      4e0 * pi * delt * d.uj[1 * V + f];
    const double e6 = +f1 * (+gfac * (-D(1, f) + D(1, E) + D(0, f) - D(0, N)) + (-U(1, f) + U(1, E) + U(0, f) - U(0, N))) -
                      4e0 * pi * delt * d.uj[2 * V + f];
#undef U
#undef D
    df[3 * V + f] = e4;
    df[4 * V + f] = e5;
    df[5 * V + f] = e6;
  }
}

void efield3d(const Dev3D& d, cudaStream_t s) { k_efield3d<<<8 * 152, 256, 0, s>>>(d); }

// ---------------------------------------------------------------------------
// energy_history sums  (3d/proj/weibel/app.f90:531-566), FP64, deterministic order
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(CG_THREADS) k_energy3d_kin(Dev3D d) {
  __shared__ double sh[CG_THREADS];
  const int isp = blockIdx.y;
  const double c = d.ph.c, rr = d.ph.r[isp];
  const int nrs = d.g.ny * d.g.nz;
  double v = 0.0;
  for (int rs = blockIdx.x; rs < nrs; rs += gridDim.x) {
    const int row = isp * nrs + rs;
    const size_t rb = (size_t)row * d.cap;
    for (int s = threadIdx.x; s < d.np2[row]; s += CG_THREADS) {
      const double a = d.A.ux[rb + s], b = d.A.uy[rb + s], e = d.A.uz[rb + s];
      const double u2 = a * a + b * b + e * e;
      v = v + rr * (sqrt(1e0 + u2 / (c * c)) - 1e0);
    }
  }
  v = block_sum(v, sh);
  if (threadIdx.x == 0) d.partials[((size_t)isp * d.nred + blockIdx.x) * 2] = v;
}

__global__ void __launch_bounds__(CG_THREADS) k_energy3d_fld(Dev3D d) {
  __shared__ double sh[CG_THREADS];
  const Grid3D g = d.g;
  double be = 0.0, ee = 0.0;
  for (size_t cid = (size_t)blockIdx.x * CG_THREADS + threadIdx.x; cid < g.ncell; cid += (size_t)gridDim.x * CG_THREADS) {
    const int cx = (int)(cid % g.nx), cy = (int)((cid / g.nx) % g.ny), cz = (int)(cid / ((size_t)g.nx * g.ny));
    const size_t f = f3(g, cx + 2, cy + 2, cz + 2);
    const double* U = d.uf;
    const size_t V = g.fvol;
    be = be + U[f] * U[f] + U[V + f] * U[V + f] + U[2 * V + f] * U[2 * V + f];
    ee = ee + U[3 * V + f] * U[3 * V + f] + U[4 * V + f] * U[4 * V + f] + U[5 * V + f] * U[5 * V + f];
  }
  be = block_sum(be, sh);
  ee = block_sum(ee, sh);
  if (threadIdx.x == 0) {
    d.partials[((size_t)2 * d.nred + blockIdx.x) * 2 + 0] = ee;
    d.partials[((size_t)2 * d.nred + blockIdx.x) * 2 + 1] = be;
  }
}

__global__ void __launch_bounds__(CG_THREADS) k_energy3d_fin(Dev3D d) {
  __shared__ double sh[CG_THREADS];
  double k0 = 0.0, k1 = 0.0, ee = 0.0, be = 0.0;
  for (int k = threadIdx.x; k < d.nred; k += CG_THREADS) {
    k0 = k0 + d.partials[((size_t)0 * d.nred + k) * 2];
    if (d.ph.nsp > 1) k1 = k1 + d.partials[((size_t)1 * d.nred + k) * 2];
    ee = ee + d.partials[((size_t)2 * d.nred + k) * 2 + 0];
    be = be + d.partials[((size_t)2 * d.nred + k) * 2 + 1];
  }
  k0 = block_sum(k0, sh);
  k1 = block_sum(k1, sh);
  ee = block_sum(ee, sh);
  be = block_sum(be, sh);
  if (threadIdx.x == 0) {
    d.red_out[0] = k0;
    d.red_out[1] = k1;
    d.red_out[2] = ee / (8e0 * d.ph.pi);
    d.red_out[3] = be / (8e0 * d.ph.pi);
  }
}

void energy3d(const Dev3D& d, cudaStream_t s) {
  cudaMemsetAsync(d.partials, 0, sizeof(double) * 2 * 3 * (size_t)d.nred, s);
  k_energy3d_kin<<<dim3(d.nred, d.ph.nsp), CG_THREADS, 0, s>>>(d);
  energy_fields_fin3d(d, s);
}

// the field sums and the final reduction, after the kinetic partials are in place
void energy_fields_fin3d(const Dev3D& d, cudaStream_t s) {
  k_energy3d_fld<<<d.nred, CG_THREADS, 0, s>>>(d);
  k_energy3d_fin<<<1, CG_THREADS, 0, s>>>(d);
}
