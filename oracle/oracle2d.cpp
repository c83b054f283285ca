// oracle2d.cpp -- CPU restatement of WumingPIC's 2D time step (TEST INFRASTRUCTURE).
//
// This file is the parity oracle for the 2D hot path.  It is used only by the
// tests, by __graft_entry__.smoke() as the checker, and by bench.py's CPU
// baseline leg.  Nothing in the product library calls it.
//
// It restates, statement for statement and in the reference's own array layout
// (Fortran column-major with the reference's lower bounds), the routines:
//   particle__solv            2d/common/particle.f90:48-179
//   ele_cur                   2d/common/field.f90:189-316
//   field__init constants     2d/common/field.f90:53-59
//   field__fdtd_i             2d/common/field.f90:66-186
//   cgm                       2d/common/field.f90:319-461
//   sort__bucket              2d/common/sort.f90:36-82
//   boundary_periodic__particle_x/_y/dfield/curre/phi
//                             2d/common/boundary_periodic.f90:61-568
//   boundary_reconnection__particle_x/dfield/curre/phi (conducting walls in x)
//                             2d/proj/reconnection/boundary_reconnection.f90:61-99,254-579
//   boundary_shock__particle_x/injection/dfield/curre/phi/mom (reflecting wall at the left,
//   the moving injection boundary at the right of the window nxs..nxe)
//                             2d/proj/shock/boundary_shock.f90:62-100,255-693
//   energy_history sums       2d/proj/weibel/app.f90:479-545
//   particle__solv_vay        2d/common/particle.f90:182-315
//   mom_calc__accl / __nvt    2d/common/mom_calc.f90:48-249
//   boundary_periodic__mom    2d/common/boundary_periodic.f90:571-636
//   boundary_reconnection__mom 2d/proj/reconnection/boundary_reconnection.f90:582-647
//
// Parity status: UNPINNED.  The reference ships no golden vectors or
// known-answer tests for this path and cannot be compiled in this image (no
// Fortran compiler, no MPI), so this restatement is checked only against
// physical invariants (charge conservation, free streaming, gyration, E x B
// drift, CG residual) in tests/.
//
// Arithmetic contract: compiled with -ffp-contract=off -frounding-math so that
// every operation is a separately rounded IEEE double operation in the
// reference's left-to-right evaluation order (gfortran -O3 without -march on
// x86-64 does not contract).  The reference switches to round-toward-minus-
// infinity inside the 2D particle boundary routines
// (2d/common/boundary_periodic.f90:74,124); this file does the same around
// those routines.  With one OpenMP thread every result, permutation and
// summation order is the single-thread reference's.
#include <cfenv>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

#pragma STDC FENV_ACCESS ON

namespace {

enum { ORC_OK = 0, ORC_CG_NOT_CONVERGED = 1, ORC_CAPACITY = 2, ORC_OUT_OF_RANGE = 3 };
enum { BC_PERIODIC = 0, BC_RECONNECTION = 1, BC_SHOCK = 2 };

struct Orc2D {
  int ndim, np, nsp, nxgs, nxge, nygs, nyge, nys, nye;
  int bc_kind;
  int nthreads;
  double delx, delt, c, gfac;
  std::vector<double> q, r;
  // field__init constants (2d/common/field.f90:53-59)
  double pi, f1, f2, f3, f4, f5, d_delx, d_delt;
  // particle__init: d_delx = 1./delx (2d/common/particle.f90:41)
  double p_d_delx;
  // SAVEd field__fdtd_i scratch (2d/common/field.f90:96-119)
  bool field_first;
  std::vector<double> df, gkl, uj;
  // SAVEd migration buffers (2d/common/boundary_periodic.f90:110-122)
  std::vector<int> flag;
  std::vector<double> bff;
  // CG control: fixed iteration counts (<0 = reference stopping rule) and last counts
  int cg_fixed[3];
  int cg_iters[3];
  int ite_max;

  // ---- index helpers (Fortran column-major, reference lower bounds) ----
  int nxw() const { return nxge - nxgs + 5; }           // nxgs-2 : nxge+2
  int nyw() const { return nye - nys + 5; }             // nys-2  : nye+2
  size_t iuf(int comp, int i, int j) const {            // uf(6, nxgs-2:nxge+2, nys-2:nye+2)
    return (size_t)(comp - 1) + 6 * ((size_t)(i - (nxgs - 2)) + (size_t)nxw() * (size_t)(j - (nys - 2)));
  }
  size_t iuj(int comp, int i, int j) const {            // uj(3, nxgs-2:nxge+2, nys-2:nye+2)
    return (size_t)(comp - 1) + 3 * ((size_t)(i - (nxgs - 2)) + (size_t)nxw() * (size_t)(j - (nys - 2)));
  }
  size_t igkl(int comp, int i, int j) const {           // gkl(3, nxgs:nxge, nys:nye)
    return (size_t)(comp - 1) + 3 * ((size_t)(i - nxgs) + (size_t)(nxge - nxgs + 1) * (size_t)(j - nys));
  }
  size_t iup(int d, int ii, int j, int isp) const {     // up(ndim, np, nys:nye, nsp)
    return (size_t)(d - 1) + (size_t)ndim * ((size_t)(ii - 1) + (size_t)np * ((size_t)(j - nys) + (size_t)(nye - nys + 1) * (size_t)(isp - 1)));
  }
  size_t icc(int i, int j, int isp) const {             // cumcnt(nxgs:nxge+1, nys:nye, nsp)
    return (size_t)(i - nxgs) + (size_t)(nxge - nxgs + 2) * ((size_t)(j - nys) + (size_t)(nye - nys + 1) * (size_t)(isp - 1));
  }
  size_t inp2(int j, int isp) const {                   // np2(nys:nye, nsp)
    return (size_t)(j - nys) + (size_t)(nye - nys + 1) * (size_t)(isp - 1);
  }
};

inline void set_threads(const Orc2D* o) {
#ifdef _OPENMP
  omp_set_num_threads(o->nthreads);
#else
  (void)o;
#endif
}

// Round-toward-minus-infinity region, applied on every OpenMP thread so that the
// multi-threaded oracle keeps the single-thread reference's arithmetic.
struct RoundDown {
  int saved;
  RoundDown() : saved(fegetround()) { fesetround(FE_DOWNWARD); }
  ~RoundDown() { fesetround(saved); }
};

// ---------------------------------------------------------------------------
// particle__solv  (2d/common/particle.f90:48-179)
// ---------------------------------------------------------------------------
// The Vay update (particle.f90:182-315, the gather shared with particle__solv): u' from
// E and the rotation at the old gamma, then gamma from the quadratic of Vay (2008).
inline void vay_update(double fac1, double fac2, double c, double bpx, double bpy, double bpz, double epx,
                       double epy, double epz, double uvm1, double uvm2, double uvm3, double* g, double* gam_out) {
  double gam = std::sqrt(c * c + uvm1 * uvm1 + uvm2 * uvm2 + uvm3 * uvm3);
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
  const double gam2 = 0.5 * (sigma + std::sqrt(sigma * sigma + 4.0 * (tau2 + ua * ua)));
  gam = std::sqrt(gam2);
  const double txxx = 1.0 / (tau2 + gam2);
  g[0] = txxx * (gam2 * uvm4 + c * ua * taux + gam * (uvm5 * tauz - uvm6 * tauy));
  g[1] = txxx * (gam2 * uvm5 + c * ua * tauy + gam * (uvm6 * taux - uvm4 * tauz));
  g[2] = txxx * (gam2 * uvm6 + c * ua * tauz + gam * (uvm4 * tauy - uvm5 * taux));
  *gam_out = 1.0 / gam;
}

// mode: PUSH_BORIS = particle__solv, PUSH_VAY = particle__solv_vay, PUSH_MOM = mom_calc__accl
// (2d/common/mom_calc.f90:48-161: the same gather and Boris rotation at half the time step,
// mom_calc__init halves delt at :36; positions copied, no move, IDs untouched).
enum { PUSH_BORIS = 0, PUSH_VAY = 1, PUSH_MOM = 2 };

int particle_solv(Orc2D* o, double* gp, const double* up, const double* uf, const int* cumcnt,
                  int nxs, int nxe, int mode = PUSH_BORIS) {
  const bool vay = mode == PUSH_VAY;
  const int nys = o->nys, nye = o->nye;
  const int tw = nxe - nxs + 3;  // tmp(1:6, nxs-1:nxe+1, nys-1:nye+1)
  std::vector<double> tmp((size_t)6 * tw * (nye - nys + 3));
  auto it = [&](int comp, int i, int j) -> double& {
    return tmp[(size_t)(comp - 1) + 6 * ((size_t)(i - (nxs - 1)) + (size_t)tw * (size_t)(j - (nys - 1)))];
  };
  set_threads(o);
  // fields at (i+1/2, j+1/2)  (particle.f90:70-83)
#pragma omp parallel for
  for (int j = nys - 1; j <= nye + 1; ++j)
    for (int i = nxs - 1; i <= nxe + 1; ++i) {
      it(1, i, j) = 0.5 * (+uf[o->iuf(1, i, j)] + uf[o->iuf(1, i, j + 1)]);
      it(2, i, j) = 0.5 * (+uf[o->iuf(2, i, j)] + uf[o->iuf(2, i + 1, j)]);
      it(3, i, j) = 0.25 * (+uf[o->iuf(3, i, j)] + uf[o->iuf(3, i + 1, j)]
                            + uf[o->iuf(3, i, j + 1)] + uf[o->iuf(3, i + 1, j + 1)]);
      it(4, i, j) = 0.5 * (+uf[o->iuf(4, i, j)] + uf[o->iuf(4, i + 1, j)]);
      it(5, i, j) = 0.5 * (+uf[o->iuf(5, i, j)] + uf[o->iuf(5, i, j + 1)]);
      it(6, i, j) = uf[o->iuf(6, i, j)];
    }

  const double d_delx = o->p_d_delx, delt = mode == PUSH_MOM ? o->delt * 0.5 : o->delt, c = o->c;
  // particle loop  (particle.f90:85-171)
#pragma omp parallel for
  for (int j = nys; j <= nye; ++j)
    for (int i = nxs; i <= nxe; ++i)
      for (int isp = 1; isp <= o->nsp; ++isp) {
        const double fac1 = o->q[isp - 1] / o->r[isp - 1] * 0.5 * delt;
        const double txxx = fac1 * fac1;
        const double fac2 = o->q[isp - 1] * delt / o->r[isp - 1];
        for (int ii = cumcnt[o->icc(i, j, isp)] + 1; ii <= cumcnt[o->icc(i + 1, j, isp)]; ++ii) {
          double sh[3][2];  // sh(-1:1, 2) -> sh[k+1][dim]
          double dh = up[o->iup(1, ii, j, isp)] * d_delx - 0.5 - i;
          sh[0][0] = 0.5 * (0.5 - dh) * (0.5 - dh);
          sh[1][0] = 0.75 - dh * dh;
          sh[2][0] = 0.5 * (0.5 + dh) * (0.5 + dh);
          dh = up[o->iup(2, ii, j, isp)] * d_delx - 0.5 - j;
          sh[0][1] = 0.5 * (0.5 - dh) * (0.5 - dh);
          sh[1][1] = 0.75 - dh * dh;
          sh[2][1] = 0.5 * (0.5 + dh) * (0.5 + dh);
          double f[6];
          for (int m = 1; m <= 6; ++m)
            f[m - 1] = +(+it(m, i - 1, j - 1) * sh[0][0] + it(m, i, j - 1) * sh[1][0] + it(m, i + 1, j - 1) * sh[2][0]) * sh[0][1]
                       + (+it(m, i - 1, j) * sh[0][0] + it(m, i, j) * sh[1][0] + it(m, i + 1, j) * sh[2][0]) * sh[1][1]
                       + (+it(m, i - 1, j + 1) * sh[0][0] + it(m, i, j + 1) * sh[1][0] + it(m, i + 1, j + 1) * sh[2][0]) * sh[2][1];
          const double bpx = f[0], bpy = f[1], bpz = f[2], epx = f[3], epy = f[4], epz = f[5];
          if (vay) {
            double g[3], igam;
            vay_update(fac1, fac2, c, bpx, bpy, bpz, epx, epy, epz, up[o->iup(3, ii, j, isp)],
                       up[o->iup(4, ii, j, isp)], up[o->iup(5, ii, j, isp)], g, &igam);
            gp[o->iup(3, ii, j, isp)] = g[0];
            gp[o->iup(4, ii, j, isp)] = g[1];
            gp[o->iup(5, ii, j, isp)] = g[2];
            gp[o->iup(1, ii, j, isp)] = up[o->iup(1, ii, j, isp)] + g[0] * delt * igam;
            gp[o->iup(2, ii, j, isp)] = up[o->iup(2, ii, j, isp)] + g[1] * delt * igam;
            continue;
          }
          // accel.
          double uvm1 = up[o->iup(3, ii, j, isp)] + fac1 * epx;
          double uvm2 = up[o->iup(4, ii, j, isp)] + fac1 * epy;
          double uvm3 = up[o->iup(5, ii, j, isp)] + fac1 * epz;
          // rotate
          double gam = std::sqrt(c * c + uvm1 * uvm1 + uvm2 * uvm2 + uvm3 * uvm3);
          const double igam = 1. / gam;
          const double fac1r = fac1 * igam;
          const double fac2r = fac2 / (gam + txxx * (bpx * bpx + bpy * bpy + bpz * bpz) * igam);
          const double uvm4 = uvm1 + fac1r * (+uvm2 * bpz - uvm3 * bpy);
          const double uvm5 = uvm2 + fac1r * (+uvm3 * bpx - uvm1 * bpz);
          const double uvm6 = uvm3 + fac1r * (+uvm1 * bpy - uvm2 * bpx);
          uvm1 = uvm1 + fac2r * (+uvm5 * bpz - uvm6 * bpy);
          uvm2 = uvm2 + fac2r * (+uvm6 * bpx - uvm4 * bpz);
          uvm3 = uvm3 + fac2r * (+uvm4 * bpy - uvm5 * bpx);
          // accel.
          const double g3 = uvm1 + fac1 * epx;
          const double g4 = uvm2 + fac1 * epy;
          const double g5 = uvm3 + fac1 * epz;
          if (mode == PUSH_MOM) {  // mom_calc.f90:154-159
            gp[o->iup(1, ii, j, isp)] = up[o->iup(1, ii, j, isp)];
            gp[o->iup(2, ii, j, isp)] = up[o->iup(2, ii, j, isp)];
          }
          gp[o->iup(3, ii, j, isp)] = g3;
          gp[o->iup(4, ii, j, isp)] = g4;
          gp[o->iup(5, ii, j, isp)] = g5;
          if (mode == PUSH_MOM) continue;
          // move
          gam = 1.0 / std::sqrt(1.0 + (+g3 * g3 + g4 * g4 + g5 * g5) / (c * c));
          gp[o->iup(1, ii, j, isp)] = up[o->iup(1, ii, j, isp)] + g3 * delt * gam;
          gp[o->iup(2, ii, j, isp)] = up[o->iup(2, ii, j, isp)] + g4 * delt * gam;
        }
      }
  // particle IDs copied wholesale (particle.f90:173-177)
  if (o->ndim == 6 && mode != PUSH_MOM) {
    const size_t n = (size_t)o->np * (nye - nys + 1) * o->nsp;
#pragma omp parallel for
    for (long long k = 0; k < (long long)n; ++k) gp[(size_t)k * 6 + 5] = up[(size_t)k * 6 + 5];
  }
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// ele_cur  (2d/common/field.f90:189-316)
// ---------------------------------------------------------------------------
int ele_cur(Orc2D* o, double* uj, const double* up, const double* gp, const int* cumcnt, int nxs, int nxe) {
  const int nys = o->nys, nye = o->nye;
  const double fac = 1.0 / 3.0;
  const double d_delx = o->d_delx, d_delt = o->d_delt, delx = o->delx, c = o->c;
  set_threads(o);
  // uj = 0 over nxs-2:nxe+2, nys-2:nye+2  (field.f90:203-205)
  for (int j = nys - 2; j <= nye + 2; ++j)
    for (int i = nxs - 2; i <= nxe + 2; ++i)
      for (int k = 1; k <= 3; ++k) uj[o->iuj(k, i, j)] = 0.0;

  const size_t nuj = (size_t)3 * o->nxw() * o->nyw();
#pragma omp parallel
  {
    // REDUCTION(+:uj): private copy, combined at the end (field.f90:209-211)
    std::vector<double> ujp(nuj, 0.0);
#pragma omp for schedule(static)
    for (int j = nys; j <= nye; ++j)
      for (int i = nxs; i <= nxe; ++i) {
        double pjx[5][5], pjy[5][5], pjz[5][5];  // p(ip,jp) -> p[ip+2][jp+2]
        for (int a = 0; a < 5; ++a)
          for (int b = 0; b < 5; ++b) pjx[a][b] = pjy[a][b] = pjz[a][b] = 0.0;
        for (int isp = 1; isp <= o->nsp; ++isp) {
          const double qs = o->q[isp - 1];
          for (int ii = cumcnt[o->icc(i, j, isp)] + 1; ii <= cumcnt[o->icc(i + 1, j, isp)]; ++ii) {
            double s0[5][2], ds[5][2];  // s0(-2:2, 2) -> s0[k+2][dim]
            double dh = up[o->iup(1, ii, j, isp)] * d_delx - 0.5 - i;
            s0[0][0] = 0.0;
            s0[1][0] = 0.5 * (0.5 - dh) * (0.5 - dh);
            s0[2][0] = 0.75 - dh * dh;
            s0[3][0] = 0.5 * (0.5 + dh) * (0.5 + dh);
            s0[4][0] = 0.0;
            dh = up[o->iup(2, ii, j, isp)] * d_delx - 0.5 - j;
            s0[0][1] = 0.0;
            s0[1][1] = 0.5 * (0.5 - dh) * (0.5 - dh);
            s0[2][1] = 0.75 - dh * dh;
            s0[3][1] = 0.5 * (0.5 + dh) * (0.5 + dh);
            s0[4][1] = 0.0;
            for (int dim = 0; dim < 2; ++dim) {
              const double xn = gp[o->iup(dim + 1, ii, j, isp)];
              const int i2 = (int)(xn * d_delx);
              dh = xn * d_delx - 0.5 - i2;
              const int inc = i2 - (dim == 0 ? i : j);
              const double s1_1 = 0.5 * (0.5 - dh) * (0.5 - dh);
              const double s1_2 = 0.75 - dh * dh;
              const double s1_3 = 0.5 * (0.5 + dh) * (0.5 + dh);
              const int ainc = std::abs(inc);
              const double smo_1 = (double)(-(inc - ainc)) * 0.5 + 0;
              const double smo_2 = (double)(-ainc + 1);
              const double smo_3 = (double)(inc + ainc) * 0.5 + 0;
              ds[0][dim] = s1_1 * smo_1;
              ds[1][dim] = s1_1 * smo_2 + s1_2 * smo_1;
              ds[2][dim] = s1_2 * smo_2 + s1_3 * smo_1 + s1_1 * smo_3;
              ds[3][dim] = s1_3 * smo_2 + s1_2 * smo_3;
              ds[4][dim] = s1_3 * smo_3;
            }
            for (int k = 0; k < 5; ++k) {
              ds[k][0] = ds[k][0] - s0[k][0];
              ds[k][1] = ds[k][1] - s0[k][1];
            }
            const double g3 = gp[o->iup(3, ii, j, isp)], g4 = gp[o->iup(4, ii, j, isp)], g5 = gp[o->iup(5, ii, j, isp)];
            const double gvz = g5 / std::sqrt(1. + (+g3 * g3 + g4 * g4 + g5 * g5) / (c * c));
            double pjtmp[5][5];
            for (int a = 0; a < 5; ++a)
              for (int b = 0; b < 5; ++b) pjtmp[a][b] = 0.0;
            for (int jp = -2; jp <= 2; ++jp)
              for (int ip = -2; ip <= 1; ++ip)
                pjtmp[ip + 3][jp + 2] = pjtmp[ip + 2][jp + 2]
                    - qs * delx * d_delt * ds[ip + 2][0] * (s0[jp + 2][1] + 0.5 * ds[jp + 2][1]);
            for (int jp = 0; jp < 5; ++jp)
              for (int ip = 0; ip < 5; ++ip) pjx[ip][jp] = pjx[ip][jp] + pjtmp[ip][jp];
            for (int a = 0; a < 5; ++a)
              for (int b = 0; b < 5; ++b) pjtmp[a][b] = 0.0;
            for (int jp = -2; jp <= 1; ++jp)
              for (int ip = -2; ip <= 2; ++ip)
                pjtmp[ip + 2][jp + 3] = pjtmp[ip + 2][jp + 2]
                    - qs * delx * d_delt * ds[jp + 2][1] * (s0[ip + 2][0] + 0.5 * ds[ip + 2][0]);
            for (int jp = 0; jp < 5; ++jp)
              for (int ip = 0; ip < 5; ++ip) pjy[ip][jp] = pjy[ip][jp] + pjtmp[ip][jp];
            for (int jp = 0; jp < 5; ++jp)
              for (int ip = 0; ip < 5; ++ip)
                pjz[ip][jp] = pjz[ip][jp]
                    + qs * gvz * (+s0[ip][0] * s0[jp][1] + 0.5 * ds[ip][0] * s0[jp][1]
                                  + 0.5 * s0[ip][0] * ds[jp][1] + fac * ds[ip][0] * ds[jp][1]);
          }
        }
        for (int jp = -2; jp <= 2; ++jp)
          for (int ip = -2; ip <= 2; ++ip) {
            ujp[o->iuj(1, i + ip, j + jp)] = ujp[o->iuj(1, i + ip, j + jp)] + pjx[ip + 2][jp + 2];
            ujp[o->iuj(2, i + ip, j + jp)] = ujp[o->iuj(2, i + ip, j + jp)] + pjy[ip + 2][jp + 2];
            ujp[o->iuj(3, i + ip, j + jp)] = ujp[o->iuj(3, i + ip, j + jp)] + pjz[ip + 2][jp + 2];
          }
      }
#pragma omp critical
    {
      for (size_t k = 0; k < nuj; ++k) uj[k] = uj[k] + ujp[k];
    }
  }
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// boundary routines for uj, df, phi (one rank: nup = ndown = 0, so every
// MPI_SENDRECV is a copy to self)
// ---------------------------------------------------------------------------

// boundary_periodic__curre (2d/common/boundary_periodic.f90:357-508);
// boundary_reconnection__curre (2d/proj/reconnection/boundary_reconnection.f90:364-502)
// is the same without the x fold and x refresh (lines 495-506).
void bc_curre(Orc2D* o, double* uj, int nxs, int nxe) {
  const int nys = o->nys, nye = o->nye;
  const int w = nxe - nxs + 5;
  std::vector<double> rcv((size_t)6 * w);
  // send rows nys-2, nys-1 to rank-1; add into nye-1, nye
  for (int i = nxs - 2; i <= nxe + 2; ++i)
    for (int k = 1; k <= 3; ++k) {
      rcv[6 * (i - (nxs - 2)) + k - 1] = uj[o->iuj(k, i, nys - 2)];
      rcv[6 * (i - (nxs - 2)) + k + 2] = uj[o->iuj(k, i, nys - 1)];
    }
  for (int i = nxs - 2; i <= nxe + 2; ++i)
    for (int k = 1; k <= 3; ++k) {
      uj[o->iuj(k, i, nye - 1)] = uj[o->iuj(k, i, nye - 1)] + rcv[6 * (i - (nxs - 2)) + k - 1];
      uj[o->iuj(k, i, nye)] = uj[o->iuj(k, i, nye)] + rcv[6 * (i - (nxs - 2)) + k + 2];
    }
  // send rows nye+1, nye+2 to rank+1; add into nys, nys+1
  for (int i = nxs - 2; i <= nxe + 2; ++i)
    for (int k = 1; k <= 3; ++k) {
      rcv[6 * (i - (nxs - 2)) + k - 1] = uj[o->iuj(k, i, nye + 1)];
      rcv[6 * (i - (nxs - 2)) + k + 2] = uj[o->iuj(k, i, nye + 2)];
    }
  for (int i = nxs - 2; i <= nxe + 2; ++i)
    for (int k = 1; k <= 3; ++k) {
      uj[o->iuj(k, i, nys)] = uj[o->iuj(k, i, nys)] + rcv[6 * (i - (nxs - 2)) + k - 1];
      uj[o->iuj(k, i, nys + 1)] = uj[o->iuj(k, i, nys + 1)] + rcv[6 * (i - (nxs - 2)) + k + 2];
    }
  // refresh ghost rows: nys, nys+1 -> nye+1, nye+2 ; nye-1, nye -> nys-2, nys-1
  for (int i = nxs - 2; i <= nxe + 2; ++i)
    for (int k = 1; k <= 3; ++k) {
      uj[o->iuj(k, i, nye + 1)] = uj[o->iuj(k, i, nys)];
      uj[o->iuj(k, i, nye + 2)] = uj[o->iuj(k, i, nys + 1)];
    }
  for (int i = nxs - 2; i <= nxe + 2; ++i)
    for (int k = 1; k <= 3; ++k) {
      uj[o->iuj(k, i, nys - 2)] = uj[o->iuj(k, i, nye - 1)];
      uj[o->iuj(k, i, nys - 1)] = uj[o->iuj(k, i, nye)];
    }
  if (o->bc_kind == BC_PERIODIC) {
    // x fold then x refresh over all rows (boundary_periodic.f90:495-506)
    for (int j = nys - 2; j <= nye + 2; ++j)
      for (int k = 1; k <= 3; ++k) uj[o->iuj(k, nxe - 1, j)] = uj[o->iuj(k, nxe - 1, j)] + uj[o->iuj(k, nxs - 2, j)];
    for (int j = nys - 2; j <= nye + 2; ++j)
      for (int k = 1; k <= 3; ++k) uj[o->iuj(k, nxe, j)] = uj[o->iuj(k, nxe, j)] + uj[o->iuj(k, nxs - 1, j)];
    for (int j = nys - 2; j <= nye + 2; ++j)
      for (int k = 1; k <= 3; ++k) uj[o->iuj(k, nxs, j)] = uj[o->iuj(k, nxs, j)] + uj[o->iuj(k, nxe + 1, j)];
    for (int j = nys - 2; j <= nye + 2; ++j)
      for (int k = 1; k <= 3; ++k) uj[o->iuj(k, nxs + 1, j)] = uj[o->iuj(k, nxs + 1, j)] + uj[o->iuj(k, nxe + 2, j)];
    for (int j = nys - 2; j <= nye + 2; ++j)
      for (int k = 1; k <= 3; ++k) {
        uj[o->iuj(k, nxs - 2, j)] = uj[o->iuj(k, nxe - 1, j)];
        uj[o->iuj(k, nxs - 1, j)] = uj[o->iuj(k, nxe, j)];
        uj[o->iuj(k, nxe + 1, j)] = uj[o->iuj(k, nxs, j)];
        uj[o->iuj(k, nxe + 2, j)] = uj[o->iuj(k, nxs + 1, j)];
      }
  }
}

// boundary_periodic__dfield (2d/common/boundary_periodic.f90:251-354);
// boundary_reconnection__dfield walls (boundary_reconnection.f90:350-358)
void bc_dfield(Orc2D* o, double* df, int nxs, int nxe) {
  const int nys = o->nys, nye = o->nye;
  // rows nys, nys+1 -> nye+1, nye+2 ; rows nye-1, nye -> nys-2, nys-1 (columns nxs:nxe)
  for (int i = nxs; i <= nxe; ++i)
    for (int k = 1; k <= 6; ++k) {
      df[o->iuf(k, i, nye + 1)] = df[o->iuf(k, i, nys)];
      df[o->iuf(k, i, nye + 2)] = df[o->iuf(k, i, nys + 1)];
    }
  for (int i = nxs; i <= nxe; ++i)
    for (int k = 1; k <= 6; ++k) {
      df[o->iuf(k, i, nys - 2)] = df[o->iuf(k, i, nye - 1)];
      df[o->iuf(k, i, nys - 1)] = df[o->iuf(k, i, nye)];
    }
  if (o->bc_kind == BC_PERIODIC) {
    for (int j = nys - 2; j <= nye + 2; ++j)
      for (int k = 1; k <= 6; ++k) df[o->iuf(k, nxs - 2, j)] = df[o->iuf(k, nxe - 1, j)];
    for (int j = nys - 2; j <= nye + 2; ++j)
      for (int k = 1; k <= 6; ++k) df[o->iuf(k, nxs - 1, j)] = df[o->iuf(k, nxe, j)];
    for (int j = nys - 2; j <= nye + 2; ++j)
      for (int k = 1; k <= 6; ++k) df[o->iuf(k, nxe + 1, j)] = df[o->iuf(k, nxs, j)];
    for (int j = nys - 2; j <= nye + 2; ++j)
      for (int k = 1; k <= 6; ++k) df[o->iuf(k, nxe + 2, j)] = df[o->iuf(k, nxs + 1, j)];
  } else {
    for (int j = nys - 2; j <= nye + 2; ++j) {
      df[o->iuf(1, nxs - 1, j)] = -df[o->iuf(1, nxs, j)];
      for (int k = 2; k <= 4; ++k) df[o->iuf(k, nxs - 1, j)] = df[o->iuf(k, nxs + 1, j)];
      for (int k = 5; k <= 6; ++k) df[o->iuf(k, nxs - 1, j)] = -df[o->iuf(k, nxs, j)];
      if (o->bc_kind == BC_SHOCK) {  // boundary_shock.f90:399-405
        for (int k = 1; k <= 6; ++k) df[o->iuf(k, nxe + 1, j)] = 0.0;
        continue;
      }
      df[o->iuf(1, nxe, j)] = -df[o->iuf(1, nxe - 1, j)];
      for (int k = 2; k <= 4; ++k) df[o->iuf(k, nxe + 1, j)] = df[o->iuf(k, nxe - 1, j)];
      for (int k = 5; k <= 6; ++k) df[o->iuf(k, nxe, j)] = -df[o->iuf(k, nxe - 1, j)];
    }
  }
}

// boundary_periodic__phi (2d/common/boundary_periodic.f90:511-568);
// boundary_reconnection__phi (boundary_reconnection.f90:505-579)
// phi(nxs-1:nxe+1, nys-1:nye+1)
void bc_phi(Orc2D* o, double* phi, int nxs, int nxe, int l) {
  const int nys = o->nys, nye = o->nye;
  const int pw = nxe - nxs + 3;
  auto P = [&](int i, int j) -> double& { return phi[(size_t)(i - (nxs - 1)) + (size_t)pw * (size_t)(j - (nys - 1))]; };
  for (int i = nxs; i <= nxe; ++i) P(i, nye + 1) = P(i, nys);
  for (int i = nxs; i <= nxe; ++i) P(i, nys - 1) = P(i, nye);
  if (o->bc_kind == BC_PERIODIC) {
    for (int j = nys - 1; j <= nye + 1; ++j) P(nxs - 1, j) = P(nxe, j);
    for (int j = nys - 1; j <= nye + 1; ++j) P(nxe + 1, j) = P(nxs, j);
  } else if (l == 1) {
    for (int j = nys - 1; j <= nye + 1; ++j) {
      P(nxs - 1, j) = -P(nxs, j);
      P(nxe + 1, j) = o->bc_kind == BC_SHOCK ? 0.0 : -P(nxe - 2, j);  // boundary_shock.f90:605-611
    }
  } else {
    for (int j = nys - 1; j <= nye + 1; ++j) {
      P(nxs - 1, j) = P(nxs + 1, j);
      P(nxe + 1, j) = o->bc_kind == BC_SHOCK ? 0.0 : P(nxe - 1, j);
    }
  }
}

// ---------------------------------------------------------------------------
// cgm  (2d/common/field.f90:319-461)
// ---------------------------------------------------------------------------
int cgm(Orc2D* o, double* db, const double* gkl, int nxs, int nxe) {
  const int nys = o->nys, nye = o->nye;
  const int pw = nxe - nxs + 3, ph = nye - nys + 3;
  const int iw = nxe - nxs + 1, ih = nye - nys + 1;
  std::vector<double> phi((size_t)pw * ph), p((size_t)pw * ph), r((size_t)iw * ih), b((size_t)iw * ih),
      ap((size_t)iw * ih);
  auto PHI = [&](int i, int j) -> double& { return phi[(size_t)(i - (nxs - 1)) + (size_t)pw * (size_t)(j - (nys - 1))]; };
  auto PP = [&](int i, int j) -> double& { return p[(size_t)(i - (nxs - 1)) + (size_t)pw * (size_t)(j - (nys - 1))]; };
  auto R = [&](int i, int j) -> double& { return r[(size_t)(i - nxs) + (size_t)iw * (size_t)(j - nys)]; };
  auto B = [&](int i, int j) -> double& { return b[(size_t)(i - nxs) + (size_t)iw * (size_t)(j - nys)]; };
  auto AP = [&](int i, int j) -> double& { return ap[(size_t)(i - nxs) + (size_t)iw * (size_t)(j - nys)]; };
  const double f4 = o->f4, f5 = o->f5, err = 1e-6;
  int status = ORC_OK;
  set_threads(o);
  for (int l = 1; l <= 3; ++l) {
    int ite = 0;
    double sum = 0.0;
#pragma omp parallel for reduction(+ : sum)
    for (int j = nys; j <= nye; ++j)
      for (int i = nxs; i <= nxe; ++i) {
        PHI(i, j) = db[o->iuf(l, i, j)];
        B(i, j) = f5 * gkl[o->igkl(l, i, j)];
        sum = sum + B(i, j) * B(i, j);
      }
    double sum_g = sum;
    const double eps = std::sqrt(sum_g) * err;
    bc_phi(o, phi.data(), nxs, nxe, l);
    double sumr = 0.0;
#pragma omp parallel for reduction(+ : sumr)
    for (int j = nys; j <= nye; ++j)
      for (int i = nxs; i <= nxe; ++i) {
        R(i, j) = B(i, j) + PHI(i, j - 1) + PHI(i - 1, j) - f4 * PHI(i, j) + PHI(i + 1, j) + PHI(i, j + 1);
        PP(i, j) = R(i, j);
        sumr = sumr + R(i, j) * R(i, j);
      }
    double sumr_g = sumr;
    const int fixed = o->cg_fixed[l - 1];
    if (fixed >= 0 || std::sqrt(sumr_g) > eps) {
      while (fixed >= 0 ? ite < fixed : sum_g > eps) {
        ite = ite + 1;
        bc_phi(o, p.data(), nxs, nxe, l);
        double sr = 0.0, sum2 = 0.0;
#pragma omp parallel for reduction(+ : sr, sum2)
        for (int j = nys; j <= nye; ++j)
          for (int i = nxs; i <= nxe; ++i) {
            AP(i, j) = -PP(i, j - 1) - PP(i - 1, j) + f4 * PP(i, j) - PP(i + 1, j) - PP(i, j + 1);
            sr = sr + R(i, j) * R(i, j);
            sum2 = sum2 + PP(i, j) * AP(i, j);
          }
        sumr_g = sr;
        const double sum2_g = sum2;
        const double av = sumr_g / sum2_g;
#pragma omp parallel for
        for (int j = nys; j <= nye; ++j)
          for (int i = nxs; i <= nxe; ++i) {
            PHI(i, j) = PHI(i, j) + av * PP(i, j);
            R(i, j) = R(i, j) - av * AP(i, j);
          }
        sum_g = std::sqrt(sumr_g);
        if (ite >= o->ite_max) {  // reference: write + stop (field.f90:427-430)
          status = ORC_CG_NOT_CONVERGED;
          break;
        }
        double sum1 = 0.0;
#pragma omp parallel for reduction(+ : sum1)
        for (int j = nys; j <= nye; ++j)
          for (int i = nxs; i <= nxe; ++i) sum1 = sum1 + R(i, j) * R(i, j);
        const double bv = sum1 / sumr_g;
#pragma omp parallel for
        for (int j = nys; j <= nye; ++j)
          for (int i = nxs; i <= nxe; ++i) PP(i, j) = R(i, j) + bv * PP(i, j);
      }
    }
    o->cg_iters[l - 1] = ite;
    for (int j = nys; j <= nye; ++j)
      for (int i = nxs; i <= nxe; ++i) db[o->iuf(l, i, j)] = PHI(i, j);
    if (status != ORC_OK) return status;
  }
  return status;
}

// ---------------------------------------------------------------------------
// field__fdtd_i  (2d/common/field.f90:66-186)
// ---------------------------------------------------------------------------
int field_fdtd_i(Orc2D* o, double* uf, const double* up, const double* gp, const int* cumcnt, int nxs, int nxe) {
  const int nys = o->nys, nye = o->nye;
  const size_t nf = (size_t)6 * o->nxw() * o->nyw();
  if (o->field_first) {
    o->df.assign(nf, 0.0);
    o->gkl.assign((size_t)3 * (o->nxge - o->nxgs + 1) * (nye - nys + 1), 0.0);
    o->uj.assign((size_t)3 * o->nxw() * o->nyw(), 0.0);
    o->field_first = false;
  }
  double* df = o->df.data();
  double* gkl = o->gkl.data();
  double* uj = o->uj.data();
  ele_cur(o, uj, up, gp, cumcnt, nxs, nxe);
  bc_curre(o, uj, nxs, nxe);
  const double f1 = o->f1, f2 = o->f2, f3 = o->f3, pi = o->pi, delt = o->delt, gfac = o->gfac;
  set_threads(o);
#pragma omp parallel for
  for (int j = nys; j <= nye; ++j)
    for (int i = nxs; i <= nxe; ++i) {
      auto U = [&](int k, int a, int b) { return uf[o->iuf(k, a, b)]; };
      auto J = [&](int k, int a, int b) { return uj[o->iuj(k, a, b)]; };
      gkl[o->igkl(1, i, j)] = +f2 * (+U(1, i, j - 1) + U(1, i - 1, j) - 4. * U(1, i, j) + U(1, i + 1, j) + U(1, i, j + 1)
                                     + f3 * (-J(3, i, j - 1) + J(3, i, j)))
                              - f1 * (-U(6, i, j - 1) + U(6, i, j));
      gkl[o->igkl(2, i, j)] = +f2 * (+U(2, i, j - 1) + U(2, i - 1, j) - 4. * U(2, i, j) + U(2, i + 1, j) + U(2, i, j + 1)
                                     - f3 * (-J(3, i - 1, j) + J(3, i, j)))
                              + f1 * (-U(6, i - 1, j) + U(6, i, j));
      gkl[o->igkl(3, i, j)] = +f2 * (+U(3, i, j - 1) + U(3, i - 1, j) - 4. * U(3, i, j) + U(3, i + 1, j) + U(3, i, j + 1)
                                     + f3 * (-J(2, i - 1, j) + J(2, i, j) + J(1, i, j - 1) - J(1, i, j)))
                              - f1 * (-U(5, i - 1, j) + U(5, i, j) + U(4, i, j - 1) - U(4, i, j));
    }
  int st = cgm(o, df, gkl, nxs, nxe);
  if (st != ORC_OK) return st;
  bc_dfield(o, df, nxs, nxe);
  set_threads(o);
#pragma omp parallel for
  for (int j = nys; j <= nye; ++j)
    for (int i = nxs; i <= nxe; ++i) {
      auto U = [&](int k, int a, int b) { return uf[o->iuf(k, a, b)]; };
      auto D = [&](int k, int a, int b) { return df[o->iuf(k, a, b)]; };
      auto J = [&](int k, int a, int b) { return uj[o->iuj(k, a, b)]; };
      const double d4 = +f1 * (+gfac * (-D(3, i, j) + D(3, i, j + 1)) + (-U(3, i, j) + U(3, i, j + 1)))
                        - 4. * pi * delt * J(1, i, j);
      const double d5 = -f1 * (+gfac * (-D(3, i, j) + D(3, i + 1, j)) + (-U(3, i, j) + U(3, i + 1, j)))
                        - 4. * pi * delt * J(2, i, j);
      const double d6 = +f1 * (+gfac * (-D(2, i, j) + D(2, i + 1, j) + D(1, i, j) - D(1, i, j + 1))
                               + (-U(2, i, j) + U(2, i + 1, j) + U(1, i, j) - U(1, i, j + 1)))
                        - 4. * pi * delt * J(3, i, j);
      df[o->iuf(4, i, j)] = d4;
      df[o->iuf(5, i, j)] = d5;
      df[o->iuf(6, i, j)] = d6;
    }
  bc_dfield(o, df, nxs, nxe);
#pragma omp parallel for
  for (int j = nys - 2; j <= nye + 2; ++j)
    for (int i = nxs - 2; i <= nxe + 2; ++i)
      for (int k = 1; k <= 6; ++k) uf[o->iuf(k, i, j)] = uf[o->iuf(k, i, j)] + df[o->iuf(k, i, j)];
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// particle boundaries
// ---------------------------------------------------------------------------

// boundary_periodic__particle_x (2d/common/boundary_periodic.f90:61-96), round down;
// boundary_reconnection__particle_x (boundary_reconnection.f90:61-99), walls in x.
int bc_particle_x(Orc2D* o, double* up, const int* np2, int nxs, int nxe) {
  const int nys = o->nys, nye = o->nye;
  const double delx = o->delx;
  set_threads(o);
  if (o->bc_kind == BC_PERIODIC) {
    for (int isp = 1; isp <= o->nsp; ++isp) {
#pragma omp parallel
      {
        RoundDown rd;
#pragma omp for
        for (int j = nys; j <= nye; ++j)
          for (int ii = 1; ii <= np2[o->inp2(j, isp)]; ++ii) {
            double& x = up[o->iup(1, ii, j, isp)];
            const int ipos = (int)(x / delx);
            if (ipos < o->nxgs)
              x = x + (double)(o->nxge - o->nxgs + 1) * delx;
            else if (ipos >= o->nxge + 1)
              x = x - (double)(o->nxge - o->nxgs + 1) * delx;
          }
      }
    }
  } else {
    for (int isp = 1; isp <= o->nsp; ++isp) {
#pragma omp parallel for
      for (int j = nys; j <= nye; ++j)
        for (int ii = 1; ii <= np2[o->inp2(j, isp)]; ++ii) {
          double& x = up[o->iup(1, ii, j, isp)];
          const int ipos = (int)(x / delx);
          if (ipos < nxs + 1) {
            x = (double)(2.0f * (float)(nxs + 1)) * delx - x;
            for (int d = 3; d <= 5; ++d) up[o->iup(d, ii, j, isp)] = -up[o->iup(d, ii, j, isp)];
          } else if (ipos >= nxe - 1) {
            x = (double)(2.0f * (float)(nxe - 1)) * delx - x;
            for (int d = 3; d <= 5; ++d) up[o->iup(d, ii, j, isp)] = -up[o->iup(d, ii, j, isp)];
          }
        }
    }
  }
  return ORC_OK;
}

// boundary_periodic__particle_y (2d/common/boundary_periodic.f90:99-248); the
// reconnection version (boundary_reconnection.f90:102-251) is identical.
// With several OpenMP threads the order inside each arrival buffer follows lock
// timing, exactly as in the reference; with one thread it is the source order.
int bc_particle_y(Orc2D* o, double* up, int* np2) {
  const int nys = o->nys, nye = o->nye, np = o->np, ndim = o->ndim;
  const int nrow = nye - nys + 1;
  if (o->flag.empty()) {
    o->flag.assign((size_t)np * nrow, 0);
    o->bff.assign((size_t)ndim * np * (nrow + 2), 0.0);
  }
  auto FLAG = [&](int k, int j) -> int& { return o->flag[(size_t)(k - 1) + (size_t)np * (size_t)(j - nys)]; };
  auto BFF = [&](int k, int j) -> double& { return o->bff[(size_t)(k - 1) + (size_t)ndim * np * (size_t)(j - (nys - 1))]; };
  const double delx = o->delx;
  int status = ORC_OK;
  std::vector<int> cnt(nrow + 2), cnt2(nrow);
  auto CNT = [&](int j) -> int& { return cnt[(size_t)(j - (nys - 1))]; };
  auto CNT2 = [&](int j) -> int& { return cnt2[(size_t)(j - nys)]; };
#ifdef _OPENMP
  std::vector<omp_lock_t> lck(nrow + 2);
  for (auto& l : lck) omp_init_lock(&l);
#endif
  set_threads(o);
  for (int isp = 1; isp <= o->nsp; ++isp) {
    std::fill(cnt.begin(), cnt.end(), 0);
    std::fill(cnt2.begin(), cnt2.end(), 0);
#pragma omp parallel
    {
      RoundDown rd;
#pragma omp for
      for (int j = nys; j <= nye; ++j)
        for (int ii = 1; ii <= np2[o->inp2(j, isp)]; ++ii) {
          const int jpos = (int)(up[o->iup(2, ii, j, isp)] / delx);
          if (jpos != j) {
            if (jpos < nys - 1 || jpos > nye + 1) {
              // beyond the ghost rows the reference writes out of bounds
#pragma omp atomic write
              status = ORC_OUT_OF_RANGE;
              continue;
            }
            if (jpos <= o->nygs - 1)
              up[o->iup(2, ii, j, isp)] = up[o->iup(2, ii, j, isp)] + (double)(o->nyge - o->nygs + 1) * delx;
            else if (jpos >= o->nyge + 1)
              up[o->iup(2, ii, j, isp)] = up[o->iup(2, ii, j, isp)] - (double)(o->nyge - o->nygs + 1) * delx;
#ifdef _OPENMP
            omp_set_lock(&lck[(size_t)(jpos - (nys - 1))]);
#endif
            for (int idim = 1; idim <= ndim; ++idim) BFF(idim + ndim * CNT(jpos), jpos) = up[o->iup(idim, ii, j, isp)];
            CNT(jpos) = CNT(jpos) + 1;
#ifdef _OPENMP
            omp_unset_lock(&lck[(size_t)(jpos - (nys - 1))]);
#endif
            CNT2(j) = CNT2(j) + 1;
            FLAG(CNT2(j), j) = ii;
          }
        }
    }
    if (status != ORC_OK) break;
    // transfer to rank-1 (self): ghost row nys-1 appended to row nye
    {
      const int cnt_tmp = CNT(nys - 1);
      for (int k = 1; k <= ndim * cnt_tmp; ++k) BFF(ndim * CNT(nye) + k, nye) = BFF(k, nys - 1);
      CNT(nye) = CNT(nye) + cnt_tmp;
    }
    // transfer to rank+1 (self): ghost row nye+1 appended to row nys
    {
      const int cnt_tmp = CNT(nye + 1);
      for (int k = 1; k <= ndim * cnt_tmp; ++k) BFF(ndim * CNT(nys) + k, nys) = BFF(k, nye + 1);
      CNT(nys) = CNT(nys) + cnt_tmp;
    }
    // fill holes (boundary_periodic.f90:193-225)
#pragma omp parallel for
    for (int j = nys; j <= nye; ++j) {
      int iii = 0;
      int cnt_tmp = CNT2(j);
      int& n2 = np2[o->inp2(j, isp)];
      for (int ii = 1; ii <= CNT2(j); ++ii) {
        if (CNT(j) == 0) {
          if (n2 < FLAG(ii, j)) break;
          bool done = false;
          while (n2 == FLAG(cnt_tmp, j)) {
            n2 = n2 - 1;
            if (n2 < FLAG(ii, j)) { done = true; break; }
            cnt_tmp = cnt_tmp - 1;
          }
          if (done) break;
          for (int idim = 1; idim <= ndim; ++idim)
            up[o->iup(idim, FLAG(ii, j), j, isp)] = up[o->iup(idim, n2, j, isp)];
          n2 = n2 - 1;
        } else {
          for (int idim = 1; idim <= ndim; ++idim)
            up[o->iup(idim, FLAG(ii, j), j, isp)] = BFF(idim + ndim * iii, j);
          iii = iii + 1;
          CNT(j) = CNT(j) - 1;
        }
      }
      if (CNT(j) > 0)
        for (int ii = 1; ii <= CNT(j); ++ii)
          for (int idim = 1; idim <= ndim; ++idim)
            up[o->iup(idim, n2 + ii, j, isp)] = BFF(ndim * iii + idim + ndim * (ii - 1), j);
    }
    for (int j = nys; j <= nye; ++j) {
      np2[o->inp2(j, isp)] = np2[o->inp2(j, isp)] + CNT(j);
      if (np2[o->inp2(j, isp)] > np) status = ORC_CAPACITY;  // reference: write + stop
    }
    if (status != ORC_OK) break;
  }
#ifdef _OPENMP
  for (auto& l : lck) omp_destroy_lock(&l);
#endif
  return status;
}

// ---------------------------------------------------------------------------
// sort__bucket  (2d/common/sort.f90:36-82)
// ---------------------------------------------------------------------------
int sort_bucket(Orc2D* o, double* gp, const double* up, int* cumcnt, const int* np2, int nxs, int nxe) {
  const int nys = o->nys, nye = o->nye, ndim = o->ndim;
  int status = ORC_OK;
  set_threads(o);
  for (int isp = 1; isp <= o->nsp; ++isp) {
#pragma omp parallel for
    for (int j = nys; j <= nye; ++j) {
      std::vector<int> cnt(nxe - nxs + 1, 0), sum_cnt(nxe - nxs + 2);
      const int n2 = np2[o->inp2(j, isp)];
      bool bad = false;
      for (int ii = 1; ii <= n2; ++ii) {
        const int i = (int)(up[o->iup(1, ii, j, isp)]);
        if (i < nxs || i > nxe) { bad = true; break; }  // reference indexes out of bounds here
        cnt[i - nxs] = cnt[i - nxs] + 1;
      }
      if (bad) {
#pragma omp atomic write
        status = ORC_OUT_OF_RANGE;
        continue;
      }
      sum_cnt[0] = 0;
      cumcnt[o->icc(nxs, j, isp)] = 0;
      for (int i = nxs + 1; i <= nxe + 1; ++i) {
        sum_cnt[i - nxs] = sum_cnt[i - 1 - nxs] + cnt[i - 1 - nxs];
        cumcnt[o->icc(i, j, isp)] = sum_cnt[i - nxs];
      }
      for (int ii = 1; ii <= n2; ++ii) {
        const int i = (int)(up[o->iup(1, ii, j, isp)]);
        for (int d = 1; d <= ndim; ++d) gp[o->iup(d, sum_cnt[i - nxs] + 1, j, isp)] = up[o->iup(d, ii, j, isp)];
        sum_cnt[i - nxs] = sum_cnt[i - nxs] + 1;
      }
    }
  }
  return status;
}

// energy_history sums (2d/proj/weibel/app.f90:502-534): out = [vene(1..nsp), E/8pi, B/8pi]
int energy(Orc2D* o, const double* up, const double* uf, const int* np2, double* out) {
  const int nys = o->nys, nye = o->nye;
  const double c = o->c;
  set_threads(o);
  for (int isp = 1; isp <= o->nsp; ++isp) {
    double vene = 0.0;
    const double rr = o->r[isp - 1];
#pragma omp parallel for reduction(+ : vene)
    for (int j = nys; j <= nye; ++j)
      for (int ii = 1; ii <= np2[o->inp2(j, isp)]; ++ii) {
        const double a = up[o->iup(3, ii, j, isp)], b = up[o->iup(4, ii, j, isp)], d = up[o->iup(5, ii, j, isp)];
        const double u2 = a * a + b * b + d * d;
        const double gam = std::sqrt(1 + u2 / (c * c));
        vene = vene + rr * (gam - 1);
      }
    out[isp - 1] = vene;
  }
  double bfield = 0.0, efield = 0.0;
#pragma omp parallel for reduction(+ : bfield, efield)
  for (int j = nys; j <= nye; ++j)
    for (int i = o->nxgs; i <= o->nxge; ++i) {
      auto U = [&](int k) { return uf[o->iuf(k, i, j)]; };
      bfield = bfield + U(1) * U(1) + U(2) * U(2) + U(3) * U(3);
      efield = efield + U(4) * U(4) + U(5) * U(5) + U(6) * U(6);
    }
  out[o->nsp] = efield / (8 * o->pi);
  out[o->nsp + 1] = bfield / (8 * o->pi);
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// boundary_shock__injection  (2d/proj/shock/boundary_shock.f90:255-297): reflection at the
// wall x = (nxs+1) dx, and at the injection boundary xend = nxe dx + v0 dt moving with the
// upstream flow u0 (four-velocity), where u_x -> 2 u0 - u_x.  Default rounding.
// ---------------------------------------------------------------------------
int bc_injection(Orc2D* o, double* up, const int* np2, int nxs, int nxe, double u0) {
  const int nys = o->nys, nye = o->nye;
  const double delx = o->delx, c = o->c, delt = o->delt;
  const double xend = nxe * delx + u0 / std::sqrt(1 + (u0 * u0) / (c * c)) * delt;
  set_threads(o);
  for (int isp = 1; isp <= o->nsp; ++isp) {
#pragma omp parallel for
    for (int j = nys; j <= nye; ++j)
      for (int ii = 1; ii <= np2[o->inp2(j, isp)]; ++ii) {
        double& x = up[o->iup(1, ii, j, isp)];
        const int ipos = (int)(x / delx);
        if (ipos < nxs + 1) {
          x = +(double)(2.0f * (float)(nxs + 1)) * delx - x;
          for (int d = 3; d <= 5; ++d) up[o->iup(d, ii, j, isp)] = -up[o->iup(d, ii, j, isp)];
        } else if (x > xend) {
          x = +2. * xend - x;
          up[o->iup(3, ii, j, isp)] = +2. * u0 - up[o->iup(3, ii, j, isp)];
          for (int d = 4; d <= 5; ++d) up[o->iup(d, ii, j, isp)] = -up[o->iup(d, ii, j, isp)];
        }
      }
  }
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// mom_calc__nvt  (2d/common/mom_calc.f90:164-249)
// mom(7, nxgs-1:nxge+1, nys-1:nye+1, nsp): number density, velocity and diagonal
// of u v at the half-integer nodes, linear (area) weights, single-thread order.
// ---------------------------------------------------------------------------
size_t imom(const Orc2D* o, int l, int i, int j, int isp) {
  const size_t nxm = (size_t)(o->nxge - o->nxgs + 3), nym = (size_t)(o->nye - o->nys + 3);
  return (size_t)(l - 1) + 7 * ((size_t)(i - (o->nxgs - 1)) + nxm * ((size_t)(j - (o->nys - 1)) + nym * (size_t)(isp - 1)));
}

int mom_nvt(Orc2D* o, double* mom, const double* up, const int* np2) {
  const size_t n = 7 * (size_t)(o->nxge - o->nxgs + 3) * (o->nye - o->nys + 3) * o->nsp;
  std::fill(mom, mom + n, 0.0);
  const double d_delx = 1.0 / o->delx, c = o->c;
  for (int isp = 1; isp <= o->nsp; ++isp)
    for (int j = o->nys; j <= o->nye; ++j)
      for (int ii = 1; ii <= np2[o->inp2(j, isp)]; ++ii) {
        const double x = up[o->iup(1, ii, j, isp)], y = up[o->iup(2, ii, j, isp)];
        const double u1 = up[o->iup(3, ii, j, isp)], u2 = up[o->iup(4, ii, j, isp)], u3 = up[o->iup(5, ii, j, isp)];
        const int ih = (int)(x * d_delx - 0.5);  // Fortran int(): truncation toward zero
        const int jh = (int)(y * d_delx - 0.5);
        if (ih < o->nxgs - 1 || ih > o->nxge || jh < o->nys - 1 || jh > o->nye) return ORC_OUT_OF_RANGE;
        const double dx = x * d_delx - 0.5 - ih, dxm = 1. - dx;
        const double dy = y * d_delx - 0.5 - jh, dym = 1. - dy;
        const double gam = 1. / std::sqrt(1.0 + (+u1 * u1 + u2 * u2 + u3 * u3) / (c * c));
        const double wx[2] = {dxm, dx}, wy[2] = {dym, dy};
        const double pre[7] = {1.0, u1 * gam, u2 * gam, u3 * gam, u1 * u1 * gam, u2 * u2 * gam, u3 * u3 * gam};
        for (int l = 1; l <= 7; ++l)
          for (int b = 0; b < 2; ++b)
            for (int a = 0; a < 2; ++a) {
              double& m = mom[imom(o, l, ih + a, jh + b, isp)];
              m = l == 1 ? m + wx[a] * wy[b] : m + pre[l - 1] * wx[a] * wy[b];
            }
      }
  return ORC_OK;
}

// boundary_periodic__mom (2d/common/boundary_periodic.f90:571-636) with one rank (the
// y exchanges are self-exchanges); boundary_reconnection__mom
// (2d/proj/reconnection/boundary_reconnection.f90:582-647) folds the x ghosts onto the
// adjacent wall columns instead of the periodic images.
void bc_mom(Orc2D* o, double* mom) {
  const int nxgs = o->nxgs, nxge = o->nxge, nys = o->nys, nye = o->nye;
  for (int isp = 1; isp <= o->nsp; ++isp)
    for (int j = nys - 1; j <= nye + 1; ++j)
      for (int l = 1; l <= 7; ++l) {
        if (o->bc_kind != BC_PERIODIC) {  // walls (reconnection, shock: boundary_shock.f90:628-693)
          mom[imom(o, l, nxgs, j, isp)] = mom[imom(o, l, nxgs, j, isp)] + mom[imom(o, l, nxgs - 1, j, isp)];
          mom[imom(o, l, nxge, j, isp)] = mom[imom(o, l, nxge, j, isp)] + mom[imom(o, l, nxge + 1, j, isp)];
        } else {
          mom[imom(o, l, nxgs, j, isp)] = mom[imom(o, l, nxgs, j, isp)] + mom[imom(o, l, nxge + 1, j, isp)];
          mom[imom(o, l, nxge, j, isp)] = mom[imom(o, l, nxge, j, isp)] + mom[imom(o, l, nxgs - 1, j, isp)];
        }
      }
  for (int isp = 1; isp <= o->nsp; ++isp) {
    for (int i = nxgs - 1; i <= nxge + 1; ++i)
      for (int l = 1; l <= 7; ++l)
        mom[imom(o, l, i, nye, isp)] = mom[imom(o, l, i, nye, isp)] + mom[imom(o, l, i, nys - 1, isp)];
    for (int i = nxgs - 1; i <= nxge + 1; ++i)
      for (int l = 1; l <= 7; ++l)
        mom[imom(o, l, i, nys, isp)] = mom[imom(o, l, i, nys, isp)] + mom[imom(o, l, i, nye + 1, isp)];
  }
}

}  // namespace

extern "C" {

void* orc2d_create(int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, int nys, int nye, double delx,
                   double delt, double c, const double* q, const double* r, double gfac, int bc_kind) {
  Orc2D* o = new Orc2D();
  o->ndim = ndim; o->np = np; o->nsp = nsp;
  o->nxgs = nxgs; o->nxge = nxge; o->nygs = nygs; o->nyge = nyge; o->nys = nys; o->nye = nye;
  o->delx = delx; o->delt = delt; o->c = c; o->gfac = gfac; o->bc_kind = bc_kind;
  o->q.assign(q, q + nsp); o->r.assign(r, r + nsp);
  o->nthreads = 1;
  o->pi = 4.0 * std::atan(1.0);
  o->f1 = c * delt / delx;
  o->f2 = gfac * o->f1 * o->f1;
  o->f3 = 4.0 * o->pi * delx / c;
  const double t = delx / (c * delt * gfac);
  o->f4 = 4.0 + t * t;
  o->f5 = t * t;
  o->d_delx = 1. / delx;
  o->d_delt = 1. / delt;
  o->p_d_delx = 1. / delx;
  o->field_first = true;
  for (int l = 0; l < 3; ++l) { o->cg_fixed[l] = -1; o->cg_iters[l] = 0; }
  o->ite_max = 100;
  return o;
}
void orc2d_destroy(void* h) { delete (Orc2D*)h; }
void orc2d_set_threads(void* h, int n) { ((Orc2D*)h)->nthreads = n > 0 ? n : 1; }
void orc2d_cg_control(void* h, const int* fixed3, int ite_max) {
  Orc2D* o = (Orc2D*)h;
  for (int l = 0; l < 3; ++l) o->cg_fixed[l] = fixed3 ? fixed3[l] : -1;
  o->ite_max = ite_max > 0 ? ite_max : 100;
}
void orc2d_cg_iters(void* h, int* out3) { for (int l = 0; l < 3; ++l) out3[l] = ((Orc2D*)h)->cg_iters[l]; }
// df / uj scratch (reference layout uf(6,...) / uj(3,...)); set_df also marks the scratch as allocated
void orc2d_get_df(void* h, double* out) {
  Orc2D* o = (Orc2D*)h;
  const size_t n = (size_t)6 * o->nxw() * o->nyw();
  if (o->df.empty()) std::memset(out, 0, n * sizeof(double)); else std::memcpy(out, o->df.data(), n * sizeof(double));
}
void orc2d_set_df(void* h, const double* in) {
  Orc2D* o = (Orc2D*)h;
  if (o->field_first) {
    o->gkl.assign((size_t)3 * (o->nxge - o->nxgs + 1) * (o->nye - o->nys + 1), 0.0);
    o->uj.assign((size_t)3 * o->nxw() * o->nyw(), 0.0);
    o->field_first = false;
  }
  o->df.assign(in, in + (size_t)6 * o->nxw() * o->nyw());
}
void orc2d_get_uj(void* h, double* out) {
  Orc2D* o = (Orc2D*)h;
  const size_t n = (size_t)3 * o->nxw() * o->nyw();
  if (o->uj.empty()) std::memset(out, 0, n * sizeof(double)); else std::memcpy(out, o->uj.data(), n * sizeof(double));
}
int orc2d_particle_solv(void* h, double* gp, const double* up, const double* uf, const int* cumcnt, int nxs, int nxe) {
  return particle_solv((Orc2D*)h, gp, up, uf, cumcnt, nxs, nxe);
}
int orc2d_particle_solv_vay(void* h, double* gp, const double* up, const double* uf, const int* cumcnt, int nxs,
                            int nxe) {
  return particle_solv((Orc2D*)h, gp, up, uf, cumcnt, nxs, nxe, PUSH_VAY);
}
int orc2d_mom_calc_accl(void* h, double* gp, const double* up, const double* uf, const int* cumcnt, int nxs,
                        int nxe) {
  return particle_solv((Orc2D*)h, gp, up, uf, cumcnt, nxs, nxe, PUSH_MOM);
}
int orc2d_mom_calc_nvt(void* h, double* mom, const double* up, const int* np2) {
  return mom_nvt((Orc2D*)h, mom, up, np2);
}
int orc2d_bc_mom(void* h, double* mom) { bc_mom((Orc2D*)h, mom); return 0; }
int orc2d_bc_injection(void* h, double* up, const int* np2, int nxs, int nxe, double u0) {
  return bc_injection((Orc2D*)h, up, np2, nxs, nxe, u0);
}
int orc2d_ele_cur(void* h, double* uj, const double* up, const double* gp, const int* cumcnt, int nxs, int nxe) {
  return ele_cur((Orc2D*)h, uj, up, gp, cumcnt, nxs, nxe);
}
int orc2d_bc_curre(void* h, double* uj, int nxs, int nxe) { bc_curre((Orc2D*)h, uj, nxs, nxe); return 0; }
int orc2d_bc_dfield(void* h, double* df, int nxs, int nxe) { bc_dfield((Orc2D*)h, df, nxs, nxe); return 0; }
int orc2d_bc_phi(void* h, double* phi, int nxs, int nxe, int l) { bc_phi((Orc2D*)h, phi, nxs, nxe, l); return 0; }
int orc2d_cgm(void* h, double* db, const double* gkl, int nxs, int nxe) { return cgm((Orc2D*)h, db, gkl, nxs, nxe); }
int orc2d_field_fdtd_i(void* h, double* uf, const double* up, const double* gp, const int* cumcnt, int nxs, int nxe) {
  return field_fdtd_i((Orc2D*)h, uf, up, gp, cumcnt, nxs, nxe);
}
int orc2d_bc_particle_x(void* h, double* up, const int* np2, int nxs, int nxe) {
  return bc_particle_x((Orc2D*)h, up, np2, nxs, nxe);
}
int orc2d_bc_particle_y(void* h, double* up, int* np2) { return bc_particle_y((Orc2D*)h, up, np2); }
int orc2d_sort_bucket(void* h, double* gp, const double* up, int* cumcnt, const int* np2, int nxs, int nxe) {
  return sort_bucket((Orc2D*)h, gp, up, cumcnt, np2, nxs, nxe);
}
int orc2d_energy(void* h, const double* up, const double* uf, const int* np2, double* out) {
  return energy((Orc2D*)h, up, uf, np2, out);
}

}  // extern "C"
