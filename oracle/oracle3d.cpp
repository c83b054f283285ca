// oracle3d.cpp -- CPU restatement of WumingPIC's 3D time step (TEST INFRASTRUCTURE).
//
// This file is the parity oracle for the 3D hot path.  It is used only by the
// tests and by __graft_entry__.smoke() / bench.py as the checker or CPU
// baseline.  Nothing in the product library calls it.
//
// It restates, statement for statement and in the reference's own array layout
// (Fortran column-major with the reference's lower bounds), the routines:
//   particle__solv            3d/common/particle.f90:52-233
//   ele_cur                   3d/common/field.f90:211-406
//   field__init constants     3d/common/field.f90:57-63
//   field__fdtd_i             3d/common/field.f90:70-208
//   cgm                       3d/common/field.f90:409-560
//   sort__bucket              3d/common/sort.f90:40-88
//   boundary_periodic__particle_x/_yz/dfield/curre/phi
//                             3d/common/boundary_periodic.f90:68-1099
//   energy_history sums       3d/proj/weibel/app.f90:509-577
//   particle__solv_vay        3d/common/particle.f90:236-419
//   mom_calc__accl / __nvt    3d/common/mom_calc.f90:49-332
//   boundary_periodic__mom    3d/common/boundary_periodic.f90:1102-1235
//   boundary_reconnection__particle_x/dfield/curre/phi/mom (conducting walls in x; its
//   particle_yz is boundary_periodic's)
//                             3d/proj/reconnection/boundary_reconnection.f90:69-1255
//   boundary_shock__injection/dfield/curre/phi/mom (wall at nxs, open end at nxe of the window)
//                             3d/proj/shock/boundary_shock.f90:424-1245
//
// Parity status: UNPINNED (no golden vectors in the reference for this path;
// no Fortran compiler or MPI in this image).  It is checked against physical
// invariants in tests/.
//
// Arithmetic contract: compiled with -ffp-contract=off -frounding-math, every
// operation a separately rounded IEEE double operation in the reference's
// left-to-right order.  The 3D particle boundaries use the default rounding
// mode (unlike 2D).  One rank: every MPI_SENDRECV is a copy to self.  With one
// OpenMP thread every result, permutation and summation order is the
// single-thread reference's.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum { ORC_OK = 0, ORC_CG_NOT_CONVERGED = 1, ORC_CAPACITY = 2, ORC_OUT_OF_RANGE = 3 };

// boundary_periodic / boundary_reconnection / boundary_shock (3D)
enum { BC3_PERIODIC = 0, BC3_WALLS = 1, BC3_SHOCK = 2 };

struct Orc3D {
  int ndim, np, nsp, nxgs, nxge, nygs, nyge, nzgs, nzge, nys, nye, nzs, nze;
  int bc_kind = BC3_PERIODIC;  // conducting walls in x (3d/proj/reconnection/boundary_reconnection.f90)
  int nthreads;
  double delx, delt, c, gfac;
  std::vector<double> q, r;
  // field__init constants (3d/common/field.f90:57-63)
  double pi, f1, f2, f3, f4, f5, d_delx, d_delt;
  // SAVEd field__fdtd_i scratch (3d/common/field.f90:104-125)
  bool field_first;
  std::vector<double> df, gkl, uj;
  // SAVEd migration buffers (3d/common/boundary_periodic.f90:117-130)
  std::vector<int> flag;
  std::vector<double> bff;
  int cg_fixed[3];
  int cg_iters[3];
  int ite_max;

  int nxw() const { return nxge - nxgs + 5; }  // nxgs-2 : nxge+2
  int nyw() const { return nye - nys + 5; }    // nys-2  : nye+2
  int nzw() const { return nze - nzs + 5; }    // nzs-2  : nze+2
  int ny() const { return nye - nys + 1; }
  int nz() const { return nze - nzs + 1; }
  size_t icell(int i, int j, int k) const {  // (nxgs-2:nxge+2, nys-2:nye+2, nzs-2:nze+2)
    return (size_t)(i - (nxgs - 2)) + (size_t)nxw() * ((size_t)(j - (nys - 2)) + (size_t)nyw() * (size_t)(k - (nzs - 2)));
  }
  size_t iuf(int comp, int i, int j, int k) const { return (size_t)(comp - 1) + 6 * icell(i, j, k); }
  size_t iuj(int comp, int i, int j, int k) const { return (size_t)(comp - 1) + 3 * icell(i, j, k); }
  size_t igkl(int comp, int i, int j, int k) const {  // gkl(3, nxgs:nxge, nys:nye, nzs:nze)
    return (size_t)(comp - 1) +
           3 * ((size_t)(i - nxgs) + (size_t)(nxge - nxgs + 1) * ((size_t)(j - nys) + (size_t)ny() * (size_t)(k - nzs)));
  }
  size_t irow(int j, int k, int isp) const {  // (nys:nye, nzs:nze, nsp)
    return (size_t)(j - nys) + (size_t)ny() * ((size_t)(k - nzs) + (size_t)nz() * (size_t)(isp - 1));
  }
  size_t iup(int d, int ii, int j, int k, int isp) const {  // up(ndim, np, nys:nye, nzs:nze, nsp)
    return (size_t)(d - 1) + (size_t)ndim * ((size_t)(ii - 1) + (size_t)np * irow(j, k, isp));
  }
  size_t icc(int i, int j, int k, int isp) const {  // cumcnt(nxgs:nxge+1, nys:nye, nzs:nze, nsp)
    return (size_t)(i - nxgs) + (size_t)(nxge - nxgs + 2) * irow(j, k, isp);
  }
  size_t inp2(int j, int k, int isp) const { return irow(j, k, isp); }
};

inline void set_threads(const Orc3D* o) {
#ifdef _OPENMP
  omp_set_num_threads(o->nthreads);
#else
  (void)o;
#endif
}

// ---------------------------------------------------------------------------
// particle__solv  (3d/common/particle.f90:52-233)
// ---------------------------------------------------------------------------
// The Vay update (3d/common/particle.f90:236-419, the gather shared with particle__solv)
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
// (3d/common/mom_calc.f90:49-216: the same gather and rotation at half the time step,
// mom_calc__init halves delt at :36; positions copied, no move, IDs untouched).
enum { PUSH_BORIS = 0, PUSH_VAY = 1, PUSH_MOM = 2 };

int particle_solv(Orc3D* o, double* gp, const double* up, const double* uf, const int* cumcnt, int nxs, int nxe,
                  int mode = PUSH_BORIS) {
  const bool vay = mode == PUSH_VAY;
  const int nys = o->nys, nye = o->nye, nzs = o->nzs, nze = o->nze;
  const int tw = nxe - nxs + 3, th = nye - nys + 3, td = nze - nzs + 3;  // tmpf(6, nxs-1:nxe+1, nys-1:nye+1, nzs-1:nze+1)
  std::vector<double> tmpf((size_t)6 * tw * th * td);
  auto T = [&](int comp, int i, int j, int k) -> double& {
    return tmpf[(size_t)(comp - 1) +
                6 * ((size_t)(i - (nxs - 1)) + (size_t)tw * ((size_t)(j - (nys - 1)) + (size_t)th * (size_t)(k - (nzs - 1))))];
  };
  auto U = [&](int comp, int i, int j, int k) { return uf[o->iuf(comp, i, j, k)]; };
  set_threads(o);
  // fields at (i+1/2, j+1/2, k+1/2)  (particle.f90:75-92)
#pragma omp parallel for
  for (int k = nzs - 1; k <= nze + 1; ++k)
    for (int j = nys - 1; j <= nye + 1; ++j)
      for (int i = nxs - 1; i <= nxe + 1; ++i) {
        T(1, i, j, k) = 2.5e-1 * (+U(1, i, j, k) + U(1, i, j + 1, k) + U(1, i, j, k + 1) + U(1, i, j + 1, k + 1));
        T(2, i, j, k) = 2.5e-1 * (+U(2, i, j, k) + U(2, i + 1, j, k) + U(2, i, j, k + 1) + U(2, i + 1, j, k + 1));
        T(3, i, j, k) = 2.5e-1 * (+U(3, i, j, k) + U(3, i + 1, j, k) + U(3, i, j + 1, k) + U(3, i + 1, j + 1, k));
        T(4, i, j, k) = 5e-1 * (+U(4, i, j, k) + U(4, i + 1, j, k));
        T(5, i, j, k) = 5e-1 * (+U(5, i, j, k) + U(5, i, j + 1, k));
        T(6, i, j, k) = 5e-1 * (+U(6, i, j, k) + U(6, i, j, k + 1));
      }
  const double d_delx = o->d_delx, delt = mode == PUSH_MOM ? o->delt * 5e-1 : o->delt, c = o->c;
#pragma omp parallel for
  for (int k = nzs; k <= nze; ++k)
    for (int j = nys; j <= nye; ++j)
      for (int i = nxs; i <= nxe; ++i)
        for (int isp = 1; isp <= o->nsp; ++isp) {
          const double fac1 = o->q[isp - 1] / o->r[isp - 1] * 5e-1 * delt;
          const double txxx = fac1 * fac1;
          const double fac2 = o->q[isp - 1] * delt / o->r[isp - 1];
          for (int ii = cumcnt[o->icc(i, j, k, isp)] + 1; ii <= cumcnt[o->icc(i + 1, j, k, isp)]; ++ii) {
            double dh = up[o->iup(1, ii, j, k, isp)] * d_delx - 5e-1 - i;
            const double shxm = 5e-1 * (5e-1 - dh) * (5e-1 - dh), shx = 7.5e-1 - dh * dh,
                         shxp = 5e-1 * (5e-1 + dh) * (5e-1 + dh);
            dh = up[o->iup(2, ii, j, k, isp)] * d_delx - 5e-1 - j;
            const double shym = 5e-1 * (5e-1 - dh) * (5e-1 - dh), shy = 7.5e-1 - dh * dh,
                         shyp = 5e-1 * (5e-1 + dh) * (5e-1 + dh);
            dh = up[o->iup(3, ii, j, k, isp)] * d_delx - 5e-1 - k;
            const double shzm = 5e-1 * (5e-1 - dh) * (5e-1 - dh), shz = 7.5e-1 - dh * dh,
                         shzp = 5e-1 * (5e-1 + dh) * (5e-1 + dh);
            // (((row(j-1)*shym + row(j)*shy) + row(j+1)*shyp)*shzm + (...)*shz) + (...)*shzp,
            // row = (t(i-1)*shxm + t(i)*shx) + t(i+1)*shxp   (particle.f90:117-177)
            auto gather = [&](int comp) {
              auto row = [&](int jj, int kk) {
                return +T(comp, i - 1, jj, kk) * shxm + T(comp, i, jj, kk) * shx + T(comp, i + 1, jj, kk) * shxp;
              };
              auto plane = [&](int kk) { return +row(j - 1, kk) * shym + row(j, kk) * shy + row(j + 1, kk) * shyp; };
              return +plane(k - 1) * shzm + plane(k) * shz + plane(k + 1) * shzp;
            };
            const double bpx = gather(1), bpy = gather(2), bpz = gather(3);
            const double epx = gather(4), epy = gather(5), epz = gather(6);
            if (vay) {
              double gg[3], igam;
              vay_update(fac1, fac2, c, bpx, bpy, bpz, epx, epy, epz, up[o->iup(4, ii, j, k, isp)],
                         up[o->iup(5, ii, j, k, isp)], up[o->iup(6, ii, j, k, isp)], gg, &igam);
              gp[o->iup(4, ii, j, k, isp)] = gg[0];
              gp[o->iup(5, ii, j, k, isp)] = gg[1];
              gp[o->iup(6, ii, j, k, isp)] = gg[2];
              gp[o->iup(1, ii, j, k, isp)] = up[o->iup(1, ii, j, k, isp)] + gg[0] * delt * igam;
              gp[o->iup(2, ii, j, k, isp)] = up[o->iup(2, ii, j, k, isp)] + gg[1] * delt * igam;
              gp[o->iup(3, ii, j, k, isp)] = up[o->iup(3, ii, j, k, isp)] + gg[2] * delt * igam;
              continue;
            }
            double uvm1 = up[o->iup(4, ii, j, k, isp)] + fac1 * epx;
            double uvm2 = up[o->iup(5, ii, j, k, isp)] + fac1 * epy;
            double uvm3 = up[o->iup(6, ii, j, k, isp)] + fac1 * epz;
            double gam = std::sqrt(c * c + uvm1 * uvm1 + uvm2 * uvm2 + uvm3 * uvm3);
            const double igam = 1e0 / gam;
            const double fac1r = fac1 * igam;
            const double fac2r = fac2 / (gam + txxx * (bpx * bpx + bpy * bpy + bpz * bpz) * igam);
            const double uvm4 = uvm1 + fac1r * (+uvm2 * bpz - uvm3 * bpy);
            const double uvm5 = uvm2 + fac1r * (+uvm3 * bpx - uvm1 * bpz);
            const double uvm6 = uvm3 + fac1r * (+uvm1 * bpy - uvm2 * bpx);
            uvm1 = uvm1 + fac2r * (+uvm5 * bpz - uvm6 * bpy);
            uvm2 = uvm2 + fac2r * (+uvm6 * bpx - uvm4 * bpz);
            uvm3 = uvm3 + fac2r * (+uvm4 * bpy - uvm5 * bpx);
            double* g = gp;
            g[o->iup(4, ii, j, k, isp)] = uvm1 + fac1 * epx;
            g[o->iup(5, ii, j, k, isp)] = uvm2 + fac1 * epy;
            g[o->iup(6, ii, j, k, isp)] = uvm3 + fac1 * epz;
            if (mode == PUSH_MOM) {  // mom_calc.f90:204-209
              g[o->iup(1, ii, j, k, isp)] = up[o->iup(1, ii, j, k, isp)];
              g[o->iup(2, ii, j, k, isp)] = up[o->iup(2, ii, j, k, isp)];
              g[o->iup(3, ii, j, k, isp)] = up[o->iup(3, ii, j, k, isp)];
              continue;
            }
            const double g4 = g[o->iup(4, ii, j, k, isp)], g5 = g[o->iup(5, ii, j, k, isp)], g6 = g[o->iup(6, ii, j, k, isp)];
            gam = 1e0 / std::sqrt(1e0 + (+g4 * g4 + g5 * g5 + g6 * g6) / (c * c));
            g[o->iup(1, ii, j, k, isp)] = up[o->iup(1, ii, j, k, isp)] + g4 * delt * gam;
            g[o->iup(2, ii, j, k, isp)] = up[o->iup(2, ii, j, k, isp)] + g5 * delt * gam;
            g[o->iup(3, ii, j, k, isp)] = up[o->iup(3, ii, j, k, isp)] + g6 * delt * gam;
          }
        }
  if (o->ndim == 7 && mode != PUSH_MOM) {
    for (int isp = 1; isp <= o->nsp; ++isp)
      for (int k = nzs; k <= nze; ++k)
        for (int j = nys; j <= nye; ++j)
          for (int ii = 1; ii <= o->np; ++ii) gp[o->iup(7, ii, j, k, isp)] = up[o->iup(7, ii, j, k, isp)];
  }
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// ele_cur  (3d/common/field.f90:211-406)
// ---------------------------------------------------------------------------
int ele_cur(Orc3D* o, double* uj, const double* up, const double* gp, const int* cumcnt, int nxs, int nxe) {
  const int nys = o->nys, nye = o->nye, nzs = o->nzs, nze = o->nze;
  const double fac = 1.0 / 3.0;
  const double d_delx = o->d_delx, d_delt = o->d_delt, delx = o->delx;
  set_threads(o);
  for (int k = nzs - 2; k <= nze + 2; ++k)
    for (int j = nys - 2; j <= nye + 2; ++j)
      for (int i = nxs - 2; i <= nxe + 2; ++i)
        for (int l = 1; l <= 3; ++l) uj[o->iuj(l, i, j, k)] = 0.0;
  const size_t nuj = (size_t)3 * o->nxw() * o->nyw() * o->nzw();
#pragma omp parallel
  {
    std::vector<double> ujp(nuj, 0.0);  // REDUCTION(+:uj) private copy
#pragma omp for schedule(static)
    for (int k = nzs; k <= nze; ++k)
      for (int j = nys; j <= nye; ++j)
        for (int i = nxs; i <= nxe; ++i) {
          double pjx[5][5][5], pjy[5][5][5], pjz[5][5][5];  // p(a,b,c) -> p[a+2][b+2][c+2]
          for (int a = 0; a < 5; ++a)
            for (int b = 0; b < 5; ++b)
              for (int cc = 0; cc < 5; ++cc) pjx[a][b][cc] = pjy[a][b][cc] = pjz[a][b][cc] = 0.0;
          for (int isp = 1; isp <= o->nsp; ++isp) {
            const double qdxdt = o->q[isp - 1] * delx * d_delt;
            for (int ii = cumcnt[o->icc(i, j, k, isp)] + 1; ii <= cumcnt[o->icc(i + 1, j, k, isp)]; ++ii) {
              double s0[3][5], ds[3][5];  // s0(dim)(-2:2)
              const int cell[3] = {i, j, k};
              for (int dim = 0; dim < 3; ++dim) {
                const double dh = up[o->iup(dim + 1, ii, j, k, isp)] * d_delx - 5e-1 - cell[dim];
                s0[dim][0] = 0e0;
                s0[dim][1] = 5e-1 * (5e-1 - dh) * (5e-1 - dh);
                s0[dim][2] = 7.5e-1 - dh * dh;
                s0[dim][3] = 5e-1 * (5e-1 + dh) * (5e-1 + dh);
                s0[dim][4] = 0e0;
              }
              for (int dim = 0; dim < 3; ++dim) {
                const double xn = gp[o->iup(dim + 1, ii, j, k, isp)];
                const int i2 = (int)(xn * d_delx);
                const double dh = xn * d_delx - 5e-1 - i2;
                const int inc = i2 - cell[dim];
                const double s1_1 = 5e-1 * (5e-1 - dh) * (5e-1 - dh);
                const double s1_2 = 7.5e-1 - dh * dh;
                const double s1_3 = 5e-1 * (5e-1 + dh) * (5e-1 + dh);
                const int ainc = std::abs(inc);
                const double smo_1 = (double)(-(inc - ainc)) * 5e-1 + 0;
                const double smo_2 = (double)(-ainc + 1);
                const double smo_3 = (double)(inc + ainc) * 5e-1 + 0;
                ds[dim][0] = s1_1 * smo_1;
                ds[dim][1] = s1_1 * smo_2 + s1_2 * smo_1;
                ds[dim][2] = s1_2 * smo_2 + s1_3 * smo_1 + s1_1 * smo_3;
                ds[dim][3] = s1_3 * smo_2 + s1_2 * smo_3;
                ds[dim][4] = s1_3 * smo_3;
              }
              for (int dim = 0; dim < 3; ++dim)
                for (int a = 0; a < 5; ++a) ds[dim][a] = ds[dim][a] - s0[dim][a];
              // (field.f90:331-381): for each (jp, kp) of the two transverse directions, the
              // prefix along the current's own direction
              for (int kp = 0; kp < 5; ++kp)
                for (int jp = 0; jp < 5; ++jp) {
                  const double* sx = s0[0];
                  const double* sy = s0[1];
                  const double* sz = s0[2];
                  const double* dx = ds[0];
                  const double* dy = ds[1];
                  const double* dz = ds[2];
                  double dstmp = ((sy[jp] + 5e-1 * dy[jp]) * sz[kp] + (5e-1 * sy[jp] + fac * dy[jp]) * dz[kp]) * qdxdt;
                  double pjtmp = -dx[0] * dstmp;
                  pjx[1][jp][kp] = pjx[1][jp][kp] + pjtmp;
                  pjtmp = pjtmp - dx[1] * dstmp;
                  pjx[2][jp][kp] = pjx[2][jp][kp] + pjtmp;
                  pjtmp = pjtmp - dx[2] * dstmp;
                  pjx[3][jp][kp] = pjx[3][jp][kp] + pjtmp;
                  pjtmp = pjtmp - dx[3] * dstmp;
                  pjx[4][jp][kp] = pjx[4][jp][kp] + pjtmp;

                  dstmp = ((sx[jp] + 5e-1 * dx[jp]) * sz[kp] + (5e-1 * sx[jp] + fac * dx[jp]) * dz[kp]) * qdxdt;
                  pjtmp = -dy[0] * dstmp;
                  pjy[1][jp][kp] = pjy[1][jp][kp] + pjtmp;
                  pjtmp = pjtmp - dy[1] * dstmp;
                  pjy[2][jp][kp] = pjy[2][jp][kp] + pjtmp;
                  pjtmp = pjtmp - dy[2] * dstmp;
                  pjy[3][jp][kp] = pjy[3][jp][kp] + pjtmp;
                  pjtmp = pjtmp - dy[3] * dstmp;
                  pjy[4][jp][kp] = pjy[4][jp][kp] + pjtmp;

                  dstmp = ((sx[jp] + 5e-1 * dx[jp]) * sy[kp] + (5e-1 * sx[jp] + fac * dx[jp]) * dy[kp]) * qdxdt;
                  pjtmp = -dz[0] * dstmp;
                  pjz[1][jp][kp] = pjz[1][jp][kp] + pjtmp;
                  pjtmp = pjtmp - dz[1] * dstmp;
                  pjz[2][jp][kp] = pjz[2][jp][kp] + pjtmp;
                  pjtmp = pjtmp - dz[2] * dstmp;
                  pjz[3][jp][kp] = pjz[3][jp][kp] + pjtmp;
                  pjtmp = pjtmp - dz[3] * dstmp;
                  pjz[4][jp][kp] = pjz[4][jp][kp] + pjtmp;
                }
            }
          }
          // flush (field.f90:391-401): pjx(ip,jp,kp), pjy(jp,ip,kp), pjz(kp,ip,jp)
          for (int kp = -2; kp <= 2; ++kp)
            for (int jp = -2; jp <= 2; ++jp)
              for (int ip = -2; ip <= 2; ++ip) {
                double* a = &ujp[o->iuj(1, i + ip, j + jp, k + kp)];
                a[0] = a[0] + pjx[ip + 2][jp + 2][kp + 2];
                a[1] = a[1] + pjy[jp + 2][ip + 2][kp + 2];
                a[2] = a[2] + pjz[kp + 2][ip + 2][jp + 2];
              }
        }
#pragma omp critical
    {
      for (size_t n = 0; n < nuj; ++n) uj[n] = uj[n] + ujp[n];
    }
  }
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// boundary_periodic__curre  (3d/common/boundary_periodic.f90:676-978)
// ---------------------------------------------------------------------------
void bc_curre(Orc3D* o, double* uj, int nxs, int nxe) {
  const int nys = o->nys, nye = o->nye, nzs = o->nzs, nze = o->nze;
  auto J = [&](int l, int i, int j, int k) -> double& { return uj[o->iuj(l, i, j, k)]; };
  // y: the ghost rows nys-2, nys-1 are sent and added into nye-1, nye (snapshot first), then
  // nye+1, nye+2 into nys, nys+1; for k over the whole ghosted range
  {
    std::vector<double> snd;
    for (int k = nzs - 2; k <= nze + 2; ++k)
      for (int i = nxs - 2; i <= nxe + 2; ++i)
        for (int l = 1; l <= 3; ++l) { snd.push_back(J(l, i, nys - 2, k)); }
    std::vector<double> snd1;
    for (int k = nzs - 2; k <= nze + 2; ++k)
      for (int i = nxs - 2; i <= nxe + 2; ++i)
        for (int l = 1; l <= 3; ++l) snd1.push_back(J(l, i, nys - 1, k));
    size_t n = 0;
    for (int k = nzs - 2; k <= nze + 2; ++k)
      for (int i = nxs - 2; i <= nxe + 2; ++i) {
        for (int l = 1; l <= 3; ++l) J(l, i, nye - 1, k) = J(l, i, nye - 1, k) + snd[n + l - 1];
        for (int l = 1; l <= 3; ++l) J(l, i, nye, k) = J(l, i, nye, k) + snd1[n + l - 1];
        n += 3;
      }
    snd.clear();
    snd1.clear();
    for (int k = nzs - 2; k <= nze + 2; ++k)
      for (int i = nxs - 2; i <= nxe + 2; ++i)
        for (int l = 1; l <= 3; ++l) {
          snd.push_back(J(l, i, nye + 1, k));
          snd1.push_back(J(l, i, nye + 2, k));
        }
    n = 0;
    for (int k = nzs - 2; k <= nze + 2; ++k)
      for (int i = nxs - 2; i <= nxe + 2; ++i) {
        for (int l = 1; l <= 3; ++l) J(l, i, nys, k) = J(l, i, nys, k) + snd[n + l - 1];
        for (int l = 1; l <= 3; ++l) J(l, i, nys + 1, k) = J(l, i, nys + 1, k) + snd1[n + l - 1];
        n += 3;
      }
  }
  // z: rows j = nys..nye only
  {
    std::vector<double> s0, s1;
    for (int j = nys; j <= nye; ++j)
      for (int i = nxs - 2; i <= nxe + 2; ++i)
        for (int l = 1; l <= 3; ++l) {
          s0.push_back(J(l, i, j, nzs - 2));
          s1.push_back(J(l, i, j, nzs - 1));
        }
    size_t n = 0;
    for (int j = nys; j <= nye; ++j)
      for (int i = nxs - 2; i <= nxe + 2; ++i) {
        for (int l = 1; l <= 3; ++l) J(l, i, j, nze - 1) = J(l, i, j, nze - 1) + s0[n + l - 1];
        for (int l = 1; l <= 3; ++l) J(l, i, j, nze) = J(l, i, j, nze) + s1[n + l - 1];
        n += 3;
      }
    s0.clear();
    s1.clear();
    for (int j = nys; j <= nye; ++j)
      for (int i = nxs - 2; i <= nxe + 2; ++i)
        for (int l = 1; l <= 3; ++l) {
          s0.push_back(J(l, i, j, nze + 1));
          s1.push_back(J(l, i, j, nze + 2));
        }
    n = 0;
    for (int j = nys; j <= nye; ++j)
      for (int i = nxs - 2; i <= nxe + 2; ++i) {
        for (int l = 1; l <= 3; ++l) J(l, i, j, nzs) = J(l, i, j, nzs) + s0[n + l - 1];
        for (int l = 1; l <= 3; ++l) J(l, i, j, nzs + 1) = J(l, i, j, nzs + 1) + s1[n + l - 1];
        n += 3;
      }
  }
  // refresh of the 1-deep margins: y for k = nzs..nze, then z for j = nys-1..nye+1
  {
    std::vector<double> s;
    for (int k = nzs; k <= nze; ++k)
      for (int i = nxs - 2; i <= nxe + 2; ++i)
        for (int l = 1; l <= 3; ++l) s.push_back(J(l, i, nys, k));
    size_t n = 0;
    for (int k = nzs; k <= nze; ++k)
      for (int i = nxs - 2; i <= nxe + 2; ++i)
        for (int l = 1; l <= 3; ++l) J(l, i, nye + 1, k) = s[n++];
    s.clear();
    for (int k = nzs; k <= nze; ++k)
      for (int i = nxs - 2; i <= nxe + 2; ++i)
        for (int l = 1; l <= 3; ++l) s.push_back(J(l, i, nye, k));
    n = 0;
    for (int k = nzs; k <= nze; ++k)
      for (int i = nxs - 2; i <= nxe + 2; ++i)
        for (int l = 1; l <= 3; ++l) J(l, i, nys - 1, k) = s[n++];
    s.clear();
    for (int j = nys - 1; j <= nye + 1; ++j)
      for (int i = nxs - 2; i <= nxe + 2; ++i)
        for (int l = 1; l <= 3; ++l) s.push_back(J(l, i, j, nzs));
    n = 0;
    for (int j = nys - 1; j <= nye + 1; ++j)
      for (int i = nxs - 2; i <= nxe + 2; ++i)
        for (int l = 1; l <= 3; ++l) J(l, i, j, nze + 1) = s[n++];
    s.clear();
    for (int j = nys - 1; j <= nye + 1; ++j)
      for (int i = nxs - 2; i <= nxe + 2; ++i)
        for (int l = 1; l <= 3; ++l) s.push_back(J(l, i, j, nze));
    n = 0;
    for (int j = nys - 1; j <= nye + 1; ++j)
      for (int i = nxs - 2; i <= nxe + 2; ++i)
        for (int l = 1; l <= 3; ++l) J(l, i, j, nzs - 1) = s[n++];
  }
  // x: fold then refresh over the whole ghosted (j, k) range, one array statement after another;
  // boundary_reconnection__curre has no x stage
  // (3d/proj/reconnection/boundary_reconnection.f90:689-978)
  // (boundary_shock__curre likewise, 3d/proj/shock/boundary_shock.f90:690-974)
  if (o->bc_kind != BC3_PERIODIC) return;
  const int jlo = nys - 2, jhi = nye + 2, klo = nzs - 2, khi = nze + 2;
  auto xstmt = [&](int dst, int src, bool add) {
    for (int k = klo; k <= khi; ++k)
      for (int j = jlo; j <= jhi; ++j)
        for (int l = 1; l <= 3; ++l)
          J(l, dst, j, k) = add ? J(l, dst, j, k) + J(l, src, j, k) : J(l, src, j, k);
  };
  xstmt(nxe - 1, nxs - 2, true);
  xstmt(nxe, nxs - 1, true);
  xstmt(nxs, nxe + 1, true);
  xstmt(nxs + 1, nxe + 2, true);
  xstmt(nxs - 2, nxe - 1, false);
  xstmt(nxs - 1, nxe, false);
  xstmt(nxe + 1, nxs, false);
  xstmt(nxe + 2, nxs + 1, false);
}

// ---------------------------------------------------------------------------
// boundary_periodic__dfield  (3d/common/boundary_periodic.f90:458-673): 2-deep ghost copies,
// y (k = nzs..nze, i = nxs..nxe), then z (j = nys-2..nye+2, i = nxs..nxe), then x (all j, k)
// ---------------------------------------------------------------------------
void bc_dfield(Orc3D* o, double* df, int nxs, int nxe) {
  const int nys = o->nys, nye = o->nye, nzs = o->nzs, nze = o->nze;
  auto D = [&](int l, int i, int j, int k) -> double& { return df[o->iuf(l, i, j, k)]; };
  std::vector<double> s;
  auto ycopy = [&](int d0, int d1, int s0, int s1) {
    s.clear();
    for (int k = nzs; k <= nze; ++k)
      for (int i = nxs; i <= nxe; ++i) {
        for (int l = 1; l <= 6; ++l) s.push_back(D(l, i, s0, k));
        for (int l = 1; l <= 6; ++l) s.push_back(D(l, i, s1, k));
      }
    size_t n = 0;
    for (int k = nzs; k <= nze; ++k)
      for (int i = nxs; i <= nxe; ++i) {
        for (int l = 1; l <= 6; ++l) D(l, i, d0, k) = s[n++];
        for (int l = 1; l <= 6; ++l) D(l, i, d1, k) = s[n++];
      }
  };
  ycopy(nye + 1, nye + 2, nys, nys + 1);
  ycopy(nys - 2, nys - 1, nye - 1, nye);
  auto zcopy = [&](int d0, int d1, int s0, int s1) {
    s.clear();
    for (int j = nys - 2; j <= nye + 2; ++j)
      for (int i = nxs; i <= nxe; ++i) {
        for (int l = 1; l <= 6; ++l) s.push_back(D(l, i, j, s0));
        for (int l = 1; l <= 6; ++l) s.push_back(D(l, i, j, s1));
      }
    size_t n = 0;
    for (int j = nys - 2; j <= nye + 2; ++j)
      for (int i = nxs; i <= nxe; ++i) {
        for (int l = 1; l <= 6; ++l) D(l, i, j, d0) = s[n++];
        for (int l = 1; l <= 6; ++l) D(l, i, j, d1) = s[n++];
      }
  };
  zcopy(nze + 1, nze + 2, nzs, nzs + 1);
  zcopy(nzs - 2, nzs - 1, nze - 1, nze);
  if (o->bc_kind == BC3_SHOCK) {
    // boundary_shock__dfield (3d/proj/shock/boundary_shock.f90:675-684): the wall at nxs as the
    // reconnection walls, every component zero in column nxe+1
    for (int k = nzs - 2; k <= nze + 2; ++k)
      for (int j = nys - 2; j <= nye + 2; ++j) {
        D(1, nxs - 1, j, k) = -D(1, nxs, j, k);
        for (int l = 2; l <= 4; ++l) D(l, nxs - 1, j, k) = D(l, nxs + 1, j, k);
        for (int l = 5; l <= 6; ++l) D(l, nxs - 1, j, k) = -D(l, nxs, j, k);
        for (int l = 1; l <= 6; ++l) D(l, nxe + 1, j, k) = 0.0;
      }
    return;
  }
  if (o->bc_kind == BC3_WALLS) {
    // boundary_reconnection__dfield's walls (3d/proj/reconnection/boundary_reconnection.f90:674-683):
    // Bx and (Ey, Ez) odd, (By, Bz, Ex) even, with the offsets of each wall; nxs-2 and nxe+2 untouched
    for (int k = nzs - 2; k <= nze + 2; ++k)
      for (int j = nys - 2; j <= nye + 2; ++j) {
        D(1, nxs - 1, j, k) = -D(1, nxs, j, k);
        for (int l = 2; l <= 4; ++l) D(l, nxs - 1, j, k) = D(l, nxs + 1, j, k);
        for (int l = 5; l <= 6; ++l) D(l, nxs - 1, j, k) = -D(l, nxs, j, k);
        D(1, nxe, j, k) = -D(1, nxe - 1, j, k);
        for (int l = 2; l <= 4; ++l) D(l, nxe + 1, j, k) = D(l, nxe - 1, j, k);
        for (int l = 5; l <= 6; ++l) D(l, nxe, j, k) = -D(l, nxe - 1, j, k);
      }
    return;
  }
  auto xstmt = [&](int dst, int src) {
    for (int k = nzs - 2; k <= nze + 2; ++k)
      for (int j = nys - 2; j <= nye + 2; ++j)
        for (int l = 1; l <= 6; ++l) D(l, dst, j, k) = D(l, src, j, k);
  };
  xstmt(nxs - 2, nxe - 1);
  xstmt(nxs - 1, nxe);
  xstmt(nxe + 1, nxs);
  xstmt(nxe + 2, nxs + 1);
}

// boundary_periodic__phi (3d/common/boundary_periodic.f90:981-1099): 1-deep copies, y (k interior,
// i interior), z (j = nys-1..nye+1, i interior), x (all j, k)
void bc_phi(Orc3D* o, double* phi, int nxs, int nxe, int l) {
  const int nys = o->nys, nye = o->nye, nzs = o->nzs, nze = o->nze;
  const int pw = nxe - nxs + 3, ph = nye - nys + 3;
  auto P = [&](int i, int j, int k) -> double& {
    return phi[(size_t)(i - (nxs - 1)) + (size_t)pw * ((size_t)(j - (nys - 1)) + (size_t)ph * (size_t)(k - (nzs - 1)))];
  };
  std::vector<double> s;
  for (int k = nzs; k <= nze; ++k)
    for (int i = nxs; i <= nxe; ++i) s.push_back(P(i, nys, k));
  size_t n = 0;
  for (int k = nzs; k <= nze; ++k)
    for (int i = nxs; i <= nxe; ++i) P(i, nye + 1, k) = s[n++];
  s.clear();
  for (int k = nzs; k <= nze; ++k)
    for (int i = nxs; i <= nxe; ++i) s.push_back(P(i, nye, k));
  n = 0;
  for (int k = nzs; k <= nze; ++k)
    for (int i = nxs; i <= nxe; ++i) P(i, nys - 1, k) = s[n++];
  s.clear();
  for (int j = nys - 1; j <= nye + 1; ++j)
    for (int i = nxs; i <= nxe; ++i) s.push_back(P(i, j, nzs));
  n = 0;
  for (int j = nys - 1; j <= nye + 1; ++j)
    for (int i = nxs; i <= nxe; ++i) P(i, j, nze + 1) = s[n++];
  s.clear();
  for (int j = nys - 1; j <= nye + 1; ++j)
    for (int i = nxs; i <= nxe; ++i) s.push_back(P(i, j, nze));
  n = 0;
  for (int j = nys - 1; j <= nye + 1; ++j)
    for (int i = nxs; i <= nxe; ++i) P(i, j, nzs - 1) = s[n++];
  if (o->bc_kind == BC3_SHOCK) {
    // boundary_shock__phi (3d/proj/shock/boundary_shock.f90:1084-1107): the wall at nxs, zero at nxe+1
    for (int k = nzs - 1; k <= nze + 1; ++k)
      for (int j = nys - 1; j <= nye + 1; ++j) {
        P(nxs - 1, j, k) = l == 1 ? -P(nxs, j, k) : P(nxs + 1, j, k);
        P(nxe + 1, j, k) = 0.0;
      }
    return;
  }
  if (o->bc_kind == BC3_WALLS) {
    // boundary_reconnection__phi (3d/proj/reconnection/boundary_reconnection.f90:1093-1117):
    // component 1 odd about nxs and nxe-1, components 2 and 3 even about nxs and nxe
    for (int k = nzs - 1; k <= nze + 1; ++k)
      for (int j = nys - 1; j <= nye + 1; ++j) {
        if (l == 1) {
          P(nxs - 1, j, k) = -P(nxs, j, k);
          P(nxe + 1, j, k) = -P(nxe - 2, j, k);
        } else {
          P(nxs - 1, j, k) = P(nxs + 1, j, k);
          P(nxe + 1, j, k) = P(nxe - 1, j, k);
        }
      }
    return;
  }
  for (int k = nzs - 1; k <= nze + 1; ++k)
    for (int j = nys - 1; j <= nye + 1; ++j) P(nxs - 1, j, k) = P(nxe, j, k);
  for (int k = nzs - 1; k <= nze + 1; ++k)
    for (int j = nys - 1; j <= nye + 1; ++j) P(nxe + 1, j, k) = P(nxs, j, k);
}

// ---------------------------------------------------------------------------
// cgm  (3d/common/field.f90:409-560)
// ---------------------------------------------------------------------------
int cgm(Orc3D* o, double* db, const double* gkl, int nxs, int nxe) {
  const int nys = o->nys, nye = o->nye, nzs = o->nzs, nze = o->nze;
  const int pw = nxe - nxs + 3, ph = nye - nys + 3, pd = nze - nzs + 3;
  const int iw = nxe - nxs + 1, ih = nye - nys + 1, id = nze - nzs + 1;
  std::vector<double> phi((size_t)pw * ph * pd), p((size_t)pw * ph * pd), r((size_t)iw * ih * id),
      b((size_t)iw * ih * id), ap((size_t)iw * ih * id);
  auto PI = [&](int i, int j, int k) {
    return (size_t)(i - (nxs - 1)) + (size_t)pw * ((size_t)(j - (nys - 1)) + (size_t)ph * (size_t)(k - (nzs - 1)));
  };
  auto II = [&](int i, int j, int k) {
    return (size_t)(i - nxs) + (size_t)iw * ((size_t)(j - nys) + (size_t)ih * (size_t)(k - nzs));
  };
  const double f4 = o->f4, f5 = o->f5, err = 1e-6;
  int status = ORC_OK;
  set_threads(o);
  for (int l = 1; l <= 3; ++l) {
    int ite = 0;
    double sum = 0.0;
#pragma omp parallel for reduction(+ : sum)
    for (int k = nzs; k <= nze; ++k)
      for (int j = nys; j <= nye; ++j)
        for (int i = nxs; i <= nxe; ++i) {
          phi[PI(i, j, k)] = db[o->iuf(l, i, j, k)];
          b[II(i, j, k)] = f5 * gkl[o->igkl(l, i, j, k)];
          sum = sum + b[II(i, j, k)] * b[II(i, j, k)];
        }
    double sum_g = sum;
    const double eps = std::sqrt(sum_g) * err;
    bc_phi(o, phi.data(), nxs, nxe, l);
    double sumr = 0.0;
#pragma omp parallel for reduction(+ : sumr)
    for (int k = nzs; k <= nze; ++k)
      for (int j = nys; j <= nye; ++j)
        for (int i = nxs; i <= nxe; ++i) {
          const double rr = b[II(i, j, k)] + phi[PI(i, j, k - 1)] + phi[PI(i, j - 1, k)] + phi[PI(i - 1, j, k)] -
                            f4 * phi[PI(i, j, k)] + phi[PI(i + 1, j, k)] + phi[PI(i, j + 1, k)] + phi[PI(i, j, k + 1)];
          r[II(i, j, k)] = rr;
          p[PI(i, j, k)] = rr;
          sumr = sumr + rr * rr;
        }
    double sumr_g = sumr;
    const int fixed = o->cg_fixed[l - 1];
    if (fixed >= 0 || std::sqrt(sumr_g) > eps) {
      while (fixed >= 0 ? ite < fixed : sum_g > eps) {
        ite = ite + 1;
        bc_phi(o, p.data(), nxs, nxe, l);
        double sr = 0.0, sum2 = 0.0;
#pragma omp parallel for reduction(+ : sr, sum2)
        for (int k = nzs; k <= nze; ++k)
          for (int j = nys; j <= nye; ++j)
            for (int i = nxs; i <= nxe; ++i) {
              const double a = -p[PI(i, j, k - 1)] - p[PI(i, j - 1, k)] - p[PI(i - 1, j, k)] + f4 * p[PI(i, j, k)] -
                               p[PI(i + 1, j, k)] - p[PI(i, j + 1, k)] - p[PI(i, j, k + 1)];
              ap[II(i, j, k)] = a;
              sr = sr + r[II(i, j, k)] * r[II(i, j, k)];
              sum2 = sum2 + p[PI(i, j, k)] * a;
            }
        sumr_g = sr;
        const double av = sumr_g / sum2;
#pragma omp parallel for
        for (int k = nzs; k <= nze; ++k)
          for (int j = nys; j <= nye; ++j)
            for (int i = nxs; i <= nxe; ++i) {
              phi[PI(i, j, k)] = phi[PI(i, j, k)] + av * p[PI(i, j, k)];
              r[II(i, j, k)] = r[II(i, j, k)] - av * ap[II(i, j, k)];
            }
        sum_g = std::sqrt(sumr_g);
        if (ite >= o->ite_max) {
          status = ORC_CG_NOT_CONVERGED;
          break;
        }
        double sum1 = 0.0;
#pragma omp parallel for reduction(+ : sum1)
        for (int k = nzs; k <= nze; ++k)
          for (int j = nys; j <= nye; ++j)
            for (int i = nxs; i <= nxe; ++i) sum1 = sum1 + r[II(i, j, k)] * r[II(i, j, k)];
        const double bv = sum1 / sumr_g;
#pragma omp parallel for
        for (int k = nzs; k <= nze; ++k)
          for (int j = nys; j <= nye; ++j)
            for (int i = nxs; i <= nxe; ++i) p[PI(i, j, k)] = r[II(i, j, k)] + bv * p[PI(i, j, k)];
      }
    }
    o->cg_iters[l - 1] = ite;
    for (int k = nzs; k <= nze; ++k)
      for (int j = nys; j <= nye; ++j)
        for (int i = nxs; i <= nxe; ++i) db[o->iuf(l, i, j, k)] = phi[PI(i, j, k)];
    if (status != ORC_OK) return status;
  }
  return status;
}

// ---------------------------------------------------------------------------
// field__fdtd_i  (3d/common/field.f90:70-208)
// ---------------------------------------------------------------------------
int field_fdtd_i(Orc3D* o, double* uf, const double* up, const double* gp, const int* cumcnt, int nxs, int nxe) {
  const int nys = o->nys, nye = o->nye, nzs = o->nzs, nze = o->nze;
  const size_t ncell = (size_t)o->nxw() * o->nyw() * o->nzw();
  if (o->field_first) {
    o->df.assign(6 * ncell, 0.0);
    o->gkl.assign((size_t)3 * (o->nxge - o->nxgs + 1) * o->ny() * o->nz(), 0.0);
    o->uj.assign(3 * ncell, 0.0);
    o->field_first = false;
  }
  double* df = o->df.data();
  double* uj = o->uj.data();
  double* gkl = o->gkl.data();
  ele_cur(o, uj, up, gp, cumcnt, nxs, nxe);
  bc_curre(o, uj, nxs, nxe);
  const double f1 = o->f1, f2 = o->f2, f3 = o->f3, gfac = o->gfac, pi = o->pi, delt = o->delt;
  auto U = [&](int l, int i, int j, int k) { return uf[o->iuf(l, i, j, k)]; };
  auto J = [&](int l, int i, int j, int k) { return uj[o->iuj(l, i, j, k)]; };
  set_threads(o);
#pragma omp parallel for
  for (int k = nzs; k <= nze; ++k)
    for (int j = nys; j <= nye; ++j)
      for (int i = nxs; i <= nxe; ++i) {
        gkl[o->igkl(1, i, j, k)] =
            +f2 * (+U(1, i, j, k - 1) + U(1, i, j - 1, k) + U(1, i - 1, j, k) - 6e0 * U(1, i, j, k) + U(1, i + 1, j, k) +
                   U(1, i, j + 1, k) + U(1, i, j, k + 1) +
                   f3 * (-J(3, i, j - 1, k) + J(3, i, j, k) + J(2, i, j, k - 1) - J(2, i, j, k))) -
            f1 * (-U(6, i, j - 1, k) + U(6, i, j, k) + U(5, i, j, k - 1) - U(5, i, j, k));
        gkl[o->igkl(2, i, j, k)] =
            +f2 * (+U(2, i, j, k - 1) + U(2, i, j - 1, k) + U(2, i - 1, j, k) - 6e0 * U(2, i, j, k) + U(2, i + 1, j, k) +
                   U(2, i, j + 1, k) + U(2, i, j, k + 1) +
                   f3 * (-J(1, i, j, k - 1) + J(1, i, j, k) + J(3, i - 1, j, k) - J(3, i, j, k))) -
            f1 * (-U(4, i, j, k - 1) + U(4, i, j, k) + U(6, i - 1, j, k) - U(6, i, j, k));
        gkl[o->igkl(3, i, j, k)] =
            +f2 * (+U(3, i, j, k - 1) + U(3, i, j - 1, k) + U(3, i - 1, j, k) - 6e0 * U(3, i, j, k) + U(3, i + 1, j, k) +
                   U(3, i, j + 1, k) + U(3, i, j, k + 1) +
                   f3 * (-J(2, i - 1, j, k) + J(2, i, j, k) + J(1, i, j - 1, k) - J(1, i, j, k))) -
            f1 * (-U(5, i - 1, j, k) + U(5, i, j, k) + U(4, i, j - 1, k) - U(4, i, j, k));
      }
  int st = cgm(o, df, gkl, nxs, nxe);
  if (st != ORC_OK) return st;
  bc_dfield(o, df, nxs, nxe);
  auto D = [&](int l, int i, int j, int k) { return df[o->iuf(l, i, j, k)]; };
#pragma omp parallel for
  for (int k = nzs; k <= nze; ++k)
    for (int j = nys; j <= nye; ++j)
      for (int i = nxs; i <= nxe; ++i) {
        df[o->iuf(4, i, j, k)] = +f1 * (+gfac * (-D(3, i, j, k) + D(3, i, j + 1, k) + D(2, i, j, k) - D(2, i, j, k + 1)) +
                                        (-U(3, i, j, k) + U(3, i, j + 1, k) + U(2, i, j, k) - U(2, i, j, k + 1))) -
                                 4e0 * pi * delt * J(1, i, j, k);
        df[o->iuf(5, i, j, k)] = +f1 * (+gfac * (-D(1, i, j, k) + D(1, i, j, k + 1) + D(3, i, j, k) - D(3, i + 1, j, k)) +
                                        (-U(1, i, j, k) + U(1, i, j, k + 1) + U(3, i, j, k) - U(3, i + 1, j, k))) -
                                 4e0 * pi * delt * J(2, i, j, k);
        df[o->iuf(6, i, j, k)] = +f1 * (+gfac * (-D(2, i, j, k) + D(2, i + 1, j, k) + D(1, i, j, k) - D(1, i, j + 1, k)) +
                                        (-U(2, i, j, k) + U(2, i + 1, j, k) + U(1, i, j, k) - U(1, i, j + 1, k))) -
                                 4e0 * pi * delt * J(3, i, j, k);
      }
  bc_dfield(o, df, nxs, nxe);
#pragma omp parallel for
  for (int k = nzs - 2; k <= nze + 2; ++k)
    for (int j = nys - 2; j <= nye + 2; ++j)
      for (int i = nxs - 2; i <= nxe + 2; ++i)
        for (int ieq = 1; ieq <= 6; ++ieq) uf[o->iuf(ieq, i, j, k)] = uf[o->iuf(ieq, i, j, k)] + D(ieq, i, j, k);
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// boundary_periodic__particle_x  (3d/common/boundary_periodic.f90:68-101), default rounding
// ---------------------------------------------------------------------------
int bc_particle_x(Orc3D* o, double* up, const int* np2) {
  const int nys = o->nys, nye = o->nye, nzs = o->nzs, nze = o->nze;
  const double d_delx = o->d_delx, delx = o->delx;
  set_threads(o);
  if (o->bc_kind == BC3_WALLS) {
    // boundary_reconnection__particle_x (3d/proj/reconnection/boundary_reconnection.f90:69-109):
    // cell int(x / dx) below nxs+1 or from nxe-1 up reflects about that face, all three momentum
    // components reversed; the driver passes nxs = nxgs, nxe = nxge
    const int nxs = o->nxgs, nxe = o->nxge;
    for (int isp = 1; isp <= o->nsp; ++isp) {
#pragma omp parallel for
      for (int k = nzs; k <= nze; ++k)
        for (int j = nys; j <= nye; ++j)
          for (int ii = 1; ii <= np2[o->inp2(j, k, isp)]; ++ii) {
            double& x = up[o->iup(1, ii, j, k, isp)];
            const int ipos = (int)(x / delx);
            double face;
            if (ipos < nxs + 1) face = 2.0 * (nxs + 1) * delx;
            else if (ipos >= nxe - 1) face = 2.0 * (nxe - 1) * delx;
            else continue;
            x = face - x;
            for (int d = 4; d <= 6; ++d) {
              double& u = up[o->iup(d, ii, j, k, isp)];
              u = -u;
            }
          }
    }
    return ORC_OK;
  }
  for (int isp = 1; isp <= o->nsp; ++isp) {
#pragma omp parallel for
    for (int k = nzs; k <= nze; ++k)
      for (int j = nys; j <= nye; ++j)
        for (int ii = 1; ii <= np2[o->inp2(j, k, isp)]; ++ii) {
          double& x = up[o->iup(1, ii, j, k, isp)];
          const int ipos = (int)(x * d_delx);
          if (ipos < o->nxgs)
            x = x + (double)(o->nxge - o->nxgs + 1) * delx;
          else if (ipos >= o->nxge + 1)
            x = x - (double)(o->nxge - o->nxgs + 1) * delx;
        }
  }
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// boundary_shock__injection (3d/proj/shock/boundary_shock.f90:424-469): reflection at the wall
// x = (nxs+1) dx, and at xend = nxe dx + v0 dt (v0 = u0 / sqrt(1 + u0^2/c^2)) with u_x -> 2 u0 - u_x
// ---------------------------------------------------------------------------
int bc_injection(Orc3D* o, double* up, const int* np2, int nxs, int nxe, double u0) {
  const int nys = o->nys, nye = o->nye, nzs = o->nzs, nze = o->nze;
  const double delx = o->delx, c = o->c, delt = o->delt, d_delx = o->d_delx;
  const double xend = nxe * delx + u0 / std::sqrt(1.0 + (u0 * u0) / (c * c)) * delt;
  set_threads(o);
  for (int isp = 1; isp <= o->nsp; ++isp) {
#pragma omp parallel for
    for (int k = nzs; k <= nze; ++k)
      for (int j = nys; j <= nye; ++j)
        for (int ii = 1; ii <= np2[o->inp2(j, k, isp)]; ++ii) {
          double& x = up[o->iup(1, ii, j, k, isp)];
          double& ux = up[o->iup(4, ii, j, k, isp)];
          double& uy = up[o->iup(5, ii, j, k, isp)];
          double& uz = up[o->iup(6, ii, j, k, isp)];
          const int ipos = (int)(x * d_delx);
          if (ipos < nxs + 1) {
            x = 2.0 * (nxs + 1) * delx - x;
            ux = -ux;
            uy = -uy;
            uz = -uz;
          } else if (x > xend) {
            x = 2.0 * xend - x;
            ux = 2.0 * u0 - ux;
            uy = -uy;
            uz = -uz;
          }
        }
  }
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// boundary_periodic__particle_yz  (3d/common/boundary_periodic.f90:104-455).  A particle whose
// (int(y/dx), int(z/dx)) differs from its row is wrapped in y and z, appended to the buffer of
// its destination row (ghost rows included), and its slot recorded as a hole.  The ghost-row
// buffers then travel (one rank: to self) y first -- for every z row including the z ghosts,
// row nys-1 appended to nye, then nye+1 appended to nys -- and then z -- for y rows nys..nye,
// nzs-1 appended to nze, then nze+1 appended to nzs.  Holes are filled as in 2D.
// ---------------------------------------------------------------------------
int bc_particle_yz(Orc3D* o, double* up, int* np2) {
  const int nys = o->nys, nye = o->nye, nzs = o->nzs, nze = o->nze, np = o->np, ndim = o->ndim;
  const int ny = o->ny(), nz = o->nz();
  const int gy = ny + 2, gz = nz + 2;  // ghosted row grid nys-1:nye+1 x nzs-1:nze+1
  if (o->flag.empty()) {
    o->flag.assign((size_t)np * ny * nz, 0);
    o->bff.assign((size_t)ndim * np * gy * gz, 0.0);
  }
  auto G = [&](int j, int k) { return (size_t)(j - (nys - 1)) + (size_t)gy * (size_t)(k - (nzs - 1)); };
  auto FLAG = [&](int n, int j, int k) -> int& {
    return o->flag[(size_t)(n - 1) + (size_t)np * ((size_t)(j - nys) + (size_t)ny * (size_t)(k - nzs))];
  };
  auto BFF = [&](int n, int j, int k) -> double& { return o->bff[(size_t)(n - 1) + (size_t)ndim * np * G(j, k)]; };
  const double d_delx = o->d_delx, delx = o->delx;
  int status = ORC_OK;
  std::vector<int> cnt((size_t)gy * gz), cnt2((size_t)ny * nz);
  auto CNT = [&](int j, int k) -> int& { return cnt[G(j, k)]; };
  auto CNT2 = [&](int j, int k) -> int& { return cnt2[(size_t)(j - nys) + (size_t)ny * (size_t)(k - nzs)]; };
#ifdef _OPENMP
  std::vector<omp_lock_t> lck((size_t)gy * gz);
  for (auto& l : lck) omp_init_lock(&l);
#endif
  set_threads(o);
  for (int isp = 1; isp <= o->nsp; ++isp) {
    std::fill(cnt.begin(), cnt.end(), 0);
    std::fill(cnt2.begin(), cnt2.end(), 0);
#pragma omp parallel for
    for (int k = nzs; k <= nze; ++k)
      for (int j = nys; j <= nye; ++j)
        for (int ii = 1; ii <= np2[o->inp2(j, k, isp)]; ++ii) {
          const int jpos = (int)(up[o->iup(2, ii, j, k, isp)] * d_delx);
          const int kpos = (int)(up[o->iup(3, ii, j, k, isp)] * d_delx);
          if (!(jpos == j && kpos == k)) {
            if (jpos < nys - 1 || jpos > nye + 1 || kpos < nzs - 1 || kpos > nze + 1) {
#pragma omp atomic write
              status = ORC_OUT_OF_RANGE;
              continue;
            }
            double& y = up[o->iup(2, ii, j, k, isp)];
            double& z = up[o->iup(3, ii, j, k, isp)];
            if (jpos <= o->nygs - 1)
              y = y + (double)(o->nyge - o->nygs + 1) * delx;
            else if (jpos >= o->nyge + 1)
              y = y - (double)(o->nyge - o->nygs + 1) * delx;
            if (kpos <= o->nzgs - 1)
              z = z + (double)(o->nzge - o->nzgs + 1) * delx;
            else if (kpos >= o->nzge + 1)
              z = z - (double)(o->nzge - o->nzgs + 1) * delx;
#ifdef _OPENMP
            omp_set_lock(&lck[G(jpos, kpos)]);
#endif
            for (int idim = 1; idim <= ndim; ++idim)
              BFF(idim + ndim * CNT(jpos, kpos), jpos, kpos) = up[o->iup(idim, ii, j, k, isp)];
            CNT(jpos, kpos) = CNT(jpos, kpos) + 1;
#ifdef _OPENMP
            omp_unset_lock(&lck[G(jpos, kpos)]);
#endif
            CNT2(j, k) = CNT2(j, k) + 1;
            FLAG(CNT2(j, k), j, k) = ii;
          }
        }
    if (status != ORC_OK) break;
    // append buffer (sj, sk) to buffer (dj, dk)
    auto move = [&](int sj, int sk, int dj, int dk) {
      const int n = CNT(sj, sk);
      for (int m = 1; m <= ndim * n; ++m) BFF(ndim * CNT(dj, dk) + m, dj, dk) = BFF(m, sj, sk);
      CNT(dj, dk) = CNT(dj, dk) + n;
    };
    for (int k = nzs - 1; k <= nze + 1; ++k) move(nys - 1, k, nye, k);
    for (int k = nzs - 1; k <= nze + 1; ++k) move(nye + 1, k, nys, k);
    for (int j = nys; j <= nye; ++j) move(j, nzs - 1, j, nze);
    for (int j = nys; j <= nye; ++j) move(j, nze + 1, j, nzs);
    // fill holes (boundary_periodic.f90:400-440)
#pragma omp parallel for
    for (int k = nzs; k <= nze; ++k)
      for (int j = nys; j <= nye; ++j) {
        int iii = 0;
        int cnt_tmp = CNT2(j, k);
        int& n2 = np2[o->inp2(j, k, isp)];
        for (int ii = 1; ii <= CNT2(j, k); ++ii) {
          if (CNT(j, k) == 0) {
            if (n2 < FLAG(ii, j, k)) break;
            bool done = false;
            while (n2 == FLAG(cnt_tmp, j, k)) {
              n2 = n2 - 1;
              if (n2 < FLAG(ii, j, k)) { done = true; break; }
              cnt_tmp = cnt_tmp - 1;
            }
            if (done) break;
            for (int idim = 1; idim <= ndim; ++idim)
              up[o->iup(idim, FLAG(ii, j, k), j, k, isp)] = up[o->iup(idim, n2, j, k, isp)];
            n2 = n2 - 1;
          } else {
            for (int idim = 1; idim <= ndim; ++idim) up[o->iup(idim, FLAG(ii, j, k), j, k, isp)] = BFF(idim + ndim * iii, j, k);
            iii = iii + 1;
            CNT(j, k) = CNT(j, k) - 1;
          }
        }
        if (CNT(j, k) > 0)
          for (int ii = 1; ii <= CNT(j, k); ++ii)
            for (int idim = 1; idim <= ndim; ++idim)
              up[o->iup(idim, n2 + ii, j, k, isp)] = BFF(ndim * iii + idim + ndim * (ii - 1), j, k);
      }
    for (int k = nzs; k <= nze; ++k)
      for (int j = nys; j <= nye; ++j) {
        np2[o->inp2(j, k, isp)] = np2[o->inp2(j, k, isp)] + CNT(j, k);
        if (np2[o->inp2(j, k, isp)] > np) status = ORC_CAPACITY;
      }
    if (status != ORC_OK) break;
  }
#ifdef _OPENMP
  for (auto& l : lck) omp_destroy_lock(&l);
#endif
  return status;
}

// ---------------------------------------------------------------------------
// sort__bucket  (3d/common/sort.f90:40-88); i = int(x) without /dx, as the reference
// ---------------------------------------------------------------------------
int sort_bucket(Orc3D* o, double* gp, const double* up, int* cumcnt, const int* np2, int nxs, int nxe) {
  const int nys = o->nys, nye = o->nye, nzs = o->nzs, nze = o->nze, ndim = o->ndim;
  int status = ORC_OK;
  set_threads(o);
  for (int isp = 1; isp <= o->nsp; ++isp) {
#pragma omp parallel for
    for (int k = nzs; k <= nze; ++k)
      for (int j = nys; j <= nye; ++j) {
        std::vector<int> cnt(nxe - nxs + 1, 0), sum_cnt(nxe - nxs + 2, 0);
        const int n = np2[o->inp2(j, k, isp)];
        bool bad = false;
        for (int ii = 1; ii <= n; ++ii) {
          const int i = (int)(up[o->iup(1, ii, j, k, isp)]);
          if (i < nxs || i > nxe) { bad = true; break; }
          cnt[i - nxs] = cnt[i - nxs] + 1;
        }
        if (bad) {
#pragma omp atomic write
          status = ORC_OUT_OF_RANGE;
          continue;
        }
        sum_cnt[0] = 0;
        cumcnt[o->icc(nxs, j, k, isp)] = 0;
        for (int i = nxs + 1; i <= nxe + 1; ++i) {
          sum_cnt[i - nxs] = sum_cnt[i - 1 - nxs] + cnt[i - 1 - nxs];
          cumcnt[o->icc(i, j, k, isp)] = sum_cnt[i - nxs];
        }
        for (int ii = 1; ii <= n; ++ii) {
          const int i = (int)(up[o->iup(1, ii, j, k, isp)]);
          for (int d = 1; d <= ndim; ++d) gp[o->iup(d, sum_cnt[i - nxs] + 1, j, k, isp)] = up[o->iup(d, ii, j, k, isp)];
          sum_cnt[i - nxs] = sum_cnt[i - nxs] + 1;
        }
      }
  }
  return status;
}

// ---------------------------------------------------------------------------
// energy_history sums  (3d/proj/weibel/app.f90:531-566)
// ---------------------------------------------------------------------------
int energy(Orc3D* o, const double* up, const double* uf, const int* np2, double* out) {
  const int nys = o->nys, nye = o->nye, nzs = o->nzs, nze = o->nze;
  const double c = o->c;
  set_threads(o);
  for (int isp = 1; isp <= o->nsp; ++isp) {
    double vene = 0.0;
    const double rr = o->r[isp - 1];
#pragma omp parallel for reduction(+ : vene)
    for (int k = nzs; k <= nze; ++k)
      for (int j = nys; j <= nye; ++j)
        for (int ii = 1; ii <= np2[o->inp2(j, k, isp)]; ++ii) {
          const double a = up[o->iup(4, ii, j, k, isp)], b = up[o->iup(5, ii, j, k, isp)], d = up[o->iup(6, ii, j, k, isp)];
          const double u2 = a * a + b * b + d * d;
          const double gam = std::sqrt(1e0 + u2 / (c * c));
          vene = vene + rr * (gam - 1e0);
        }
    out[isp - 1] = vene;
  }
  double bfield = 0.0, efield = 0.0;
#pragma omp parallel for reduction(+ : bfield, efield)
  for (int k = nzs; k <= nze; ++k)
    for (int j = nys; j <= nye; ++j)
      for (int i = o->nxgs; i <= o->nxge; ++i) {
        auto U = [&](int l) { return uf[o->iuf(l, i, j, k)]; };
        bfield = bfield + U(1) * U(1) + U(2) * U(2) + U(3) * U(3);
        efield = efield + U(4) * U(4) + U(5) * U(5) + U(6) * U(6);
      }
  out[o->nsp] = efield / (8e0 * o->pi);
  out[o->nsp + 1] = bfield / (8e0 * o->pi);
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// mom_calc__nvt  (3d/common/mom_calc.f90:219-332)
// mom(7, nxgs-1:nxge+1, nys-1:nye+1, nzs-1:nze+1, nsp); floor() for the node index and
// the offset taken without d_delx, as the 3D reference writes them (:242-251).
// ---------------------------------------------------------------------------
size_t imom(const Orc3D* o, int l, int i, int j, int k, int isp) {
  const size_t nxm = (size_t)(o->nxge - o->nxgs + 3), nym = (size_t)(o->nye - o->nys + 3),
               nzm = (size_t)(o->nze - o->nzs + 3);
  return (size_t)(l - 1) +
         7 * ((size_t)(i - (o->nxgs - 1)) +
              nxm * ((size_t)(j - (o->nys - 1)) + nym * ((size_t)(k - (o->nzs - 1)) + nzm * (size_t)(isp - 1))));
}

int mom_nvt(Orc3D* o, double* mom, const double* up, const int* np2) {
  const size_t n = 7 * (size_t)(o->nxge - o->nxgs + 3) * (o->nye - o->nys + 3) * (o->nze - o->nzs + 3) * o->nsp;
  std::fill(mom, mom + n, 0.0);
  const double d_delx = 1e0 / o->delx, c = o->c;
  for (int isp = 1; isp <= o->nsp; ++isp)
    for (int k = o->nzs; k <= o->nze; ++k)
      for (int j = o->nys; j <= o->nye; ++j)
        for (int ii = 1; ii <= np2[o->inp2(j, k, isp)]; ++ii) {
          const double x = up[o->iup(1, ii, j, k, isp)], y = up[o->iup(2, ii, j, k, isp)],
                       z = up[o->iup(3, ii, j, k, isp)];
          const double u1 = up[o->iup(4, ii, j, k, isp)], u2 = up[o->iup(5, ii, j, k, isp)],
                       u3 = up[o->iup(6, ii, j, k, isp)];
          const int ih = (int)std::floor(x * d_delx - 5e-1);
          const int jh = (int)std::floor(y * d_delx - 5e-1);
          const int kh = (int)std::floor(z * d_delx - 5e-1);
          if (ih < o->nxgs - 1 || ih > o->nxge || jh < o->nys - 1 || jh > o->nye || kh < o->nzs - 1 || kh > o->nze)
            return ORC_OUT_OF_RANGE;
          const double dx = x - 5e-1 - ih, dxm = 1e0 - dx;
          const double dy = y - 5e-1 - jh, dym = 1e0 - dy;
          const double dz = z - 5e-1 - kh, dzm = 1e0 - dz;
          const double gam = 1e0 / std::sqrt(1e0 + (+u1 * u1 + u2 * u2 + u3 * u3) / (c * c));
          const double wx[2] = {dxm, dx}, wy[2] = {dym, dy}, wz[2] = {dzm, dz};
          const double pre[7] = {1.0, u1 * gam, u2 * gam, u3 * gam, u1 * u1 * gam, u2 * u2 * gam, u3 * u3 * gam};
          for (int l = 1; l <= 7; ++l)
            for (int cz = 0; cz < 2; ++cz)
              for (int b = 0; b < 2; ++b)
                for (int a = 0; a < 2; ++a) {
                  double& m = mom[imom(o, l, ih + a, jh + b, kh + cz, isp)];
                  m = l == 1 ? m + wx[a] * wy[b] * wz[cz] : m + pre[l - 1] * wx[a] * wy[b] * wz[cz];
                }
        }
  return ORC_OK;
}

// boundary_periodic__mom (3d/common/boundary_periodic.f90:1102-1235), one rank: x images,
// then the y self-exchange over every z layer, then the z self-exchange over the interior
// y rows.
void bc_mom(Orc3D* o, double* mom) {
  const int nxgs = o->nxgs, nxge = o->nxge, nys = o->nys, nye = o->nye, nzs = o->nzs, nze = o->nze;
  auto M = [&](int l, int i, int j, int k, int isp) -> double& { return mom[imom(o, l, i, j, k, isp)]; };
  for (int isp = 1; isp <= o->nsp; ++isp)
    for (int k = nzs - 1; k <= nze + 1; ++k)
      for (int j = nys - 1; j <= nye + 1; ++j)
        for (int l = 1; l <= 7; ++l) {
          if (o->bc_kind != BC3_PERIODIC) {  // boundary_reconnection__mom (:1134-1137), boundary_shock__mom
                                             // (3d/proj/shock/boundary_shock.f90:1124-1127): x ghosts onto the
                                             // edge columns
            M(l, nxgs, j, k, isp) = M(l, nxgs, j, k, isp) + M(l, nxgs - 1, j, k, isp);
            M(l, nxge, j, k, isp) = M(l, nxge, j, k, isp) + M(l, nxge + 1, j, k, isp);
          } else {
            M(l, nxgs, j, k, isp) = M(l, nxgs, j, k, isp) + M(l, nxge + 1, j, k, isp);
            M(l, nxge, j, k, isp) = M(l, nxge, j, k, isp) + M(l, nxgs - 1, j, k, isp);
          }
        }
  for (int isp = 1; isp <= o->nsp; ++isp) {
    for (int k = nzs - 1; k <= nze + 1; ++k)
      for (int i = nxgs - 1; i <= nxge + 1; ++i)
        for (int l = 1; l <= 7; ++l) M(l, i, nye, k, isp) = M(l, i, nye, k, isp) + M(l, i, nys - 1, k, isp);
    for (int k = nzs - 1; k <= nze + 1; ++k)
      for (int i = nxgs - 1; i <= nxge + 1; ++i)
        for (int l = 1; l <= 7; ++l) M(l, i, nys, k, isp) = M(l, i, nys, k, isp) + M(l, i, nye + 1, k, isp);
    for (int j = nys; j <= nye; ++j)
      for (int i = nxgs - 1; i <= nxge + 1; ++i)
        for (int l = 1; l <= 7; ++l) M(l, i, j, nze, isp) = M(l, i, j, nze, isp) + M(l, i, j, nzs - 1, isp);
    for (int j = nys; j <= nye; ++j)
      for (int i = nxgs - 1; i <= nxge + 1; ++i)
        for (int l = 1; l <= 7; ++l) M(l, i, j, nzs, isp) = M(l, i, j, nzs, isp) + M(l, i, j, nze + 1, isp);
  }
}

}  // namespace

extern "C" {

void* orc3d_create(int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, int nzgs, int nzge, int nys,
                   int nye, int nzs, int nze, double delx, double delt, double c, const double* q, const double* r,
                   double gfac) {
  Orc3D* o = new Orc3D();
  o->ndim = ndim; o->np = np; o->nsp = nsp;
  o->nxgs = nxgs; o->nxge = nxge; o->nygs = nygs; o->nyge = nyge; o->nzgs = nzgs; o->nzge = nzge;
  o->nys = nys; o->nye = nye; o->nzs = nzs; o->nze = nze;
  o->delx = delx; o->delt = delt; o->c = c; o->gfac = gfac;
  o->q.assign(q, q + nsp); o->r.assign(r, r + nsp);
  o->nthreads = 1;
  o->pi = 4.0 * std::atan(1.0);
  o->f1 = c * delt / delx;
  o->f2 = gfac * o->f1 * o->f1;
  o->f3 = 4.0 * o->pi * delx / c;
  const double t = delx / (c * delt * gfac);
  o->f4 = 6.0 + t * t;
  o->f5 = t * t;
  o->d_delx = 1. / delx;
  o->d_delt = 1. / delt;
  o->field_first = true;
  for (int l = 0; l < 3; ++l) { o->cg_fixed[l] = -1; o->cg_iters[l] = 0; }
  o->ite_max = 100;
  return o;
}
void orc3d_destroy(void* h) { delete (Orc3D*)h; }
void orc3d_set_bc(void* h, int bc_kind) {
  ((Orc3D*)h)->bc_kind = (bc_kind == BC3_WALLS || bc_kind == BC3_SHOCK) ? bc_kind : BC3_PERIODIC;
}
int orc3d_bc_injection(void* h, double* up, const int* np2, int nxs, int nxe, double u0) {
  return bc_injection((Orc3D*)h, up, np2, nxs, nxe, u0);
}
void orc3d_set_threads(void* h, int n) { ((Orc3D*)h)->nthreads = n > 0 ? n : 1; }
void orc3d_cg_control(void* h, const int* fixed3, int ite_max) {
  Orc3D* o = (Orc3D*)h;
  for (int l = 0; l < 3; ++l) o->cg_fixed[l] = fixed3 ? fixed3[l] : -1;
  o->ite_max = ite_max > 0 ? ite_max : 100;
}
void orc3d_cg_iters(void* h, int* out3) { for (int l = 0; l < 3; ++l) out3[l] = ((Orc3D*)h)->cg_iters[l]; }
void orc3d_get_df(void* h, double* out) {
  Orc3D* o = (Orc3D*)h;
  const size_t n = (size_t)6 * o->nxw() * o->nyw() * o->nzw();
  if (o->df.empty()) std::memset(out, 0, n * sizeof(double)); else std::memcpy(out, o->df.data(), n * sizeof(double));
}
void orc3d_get_uj(void* h, double* out) {
  Orc3D* o = (Orc3D*)h;
  const size_t n = (size_t)3 * o->nxw() * o->nyw() * o->nzw();
  if (o->uj.empty()) std::memset(out, 0, n * sizeof(double)); else std::memcpy(out, o->uj.data(), n * sizeof(double));
}
int orc3d_particle_solv(void* h, double* gp, const double* up, const double* uf, const int* cumcnt, int nxs, int nxe) {
  return particle_solv((Orc3D*)h, gp, up, uf, cumcnt, nxs, nxe);
}
int orc3d_particle_solv_vay(void* h, double* gp, const double* up, const double* uf, const int* cumcnt, int nxs,
                            int nxe) {
  return particle_solv((Orc3D*)h, gp, up, uf, cumcnt, nxs, nxe, PUSH_VAY);
}
int orc3d_mom_calc_accl(void* h, double* gp, const double* up, const double* uf, const int* cumcnt, int nxs,
                        int nxe) {
  return particle_solv((Orc3D*)h, gp, up, uf, cumcnt, nxs, nxe, PUSH_MOM);
}
int orc3d_mom_calc_nvt(void* h, double* mom, const double* up, const int* np2) {
  return mom_nvt((Orc3D*)h, mom, up, np2);
}
int orc3d_bc_mom(void* h, double* mom) {
  bc_mom((Orc3D*)h, mom);
  return 0;
}
int orc3d_ele_cur(void* h, double* uj, const double* up, const double* gp, const int* cumcnt, int nxs, int nxe) {
  return ele_cur((Orc3D*)h, uj, up, gp, cumcnt, nxs, nxe);
}
int orc3d_bc_curre(void* h, double* uj, int nxs, int nxe) { bc_curre((Orc3D*)h, uj, nxs, nxe); return 0; }
int orc3d_bc_dfield(void* h, double* df, int nxs, int nxe) { bc_dfield((Orc3D*)h, df, nxs, nxe); return 0; }
int orc3d_field_fdtd_i(void* h, double* uf, const double* up, const double* gp, const int* cumcnt, int nxs, int nxe) {
  return field_fdtd_i((Orc3D*)h, uf, up, gp, cumcnt, nxs, nxe);
}
int orc3d_bc_particle_x(void* h, double* up, const int* np2) { return bc_particle_x((Orc3D*)h, up, np2); }
int orc3d_bc_particle_yz(void* h, double* up, int* np2) { return bc_particle_yz((Orc3D*)h, up, np2); }
int orc3d_sort_bucket(void* h, double* gp, const double* up, int* cumcnt, const int* np2, int nxs, int nxe) {
  return sort_bucket((Orc3D*)h, gp, up, cumcnt, np2, nxs, nxe);
}
int orc3d_energy(void* h, const double* up, const double* uf, const int* np2, double* out) {
  return energy((Orc3D*)h, up, uf, np2, out);
}

}  // extern "C"
