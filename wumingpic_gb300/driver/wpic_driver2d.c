/* wpic_driver2d.c -- the 2D Weibel driver's main loop over the C ABI, as a compiled program.
 *
 * It calls the library in the order of the reference driver (2d/proj/weibel/app.f90:99-126):
 * every step particle__solv, field__fdtd_i, bc__particle_x, bc__particle_y, sort__bucket;
 * every intvl_mom steps mom_calc__accl, mom_calc__nvt, bc__mom and energy_history.  The host
 * arrays are brought up to date only where the driver reads them -- on entry to the diagnostic
 * block (up, np2, cumcnt and uf), which is the sync point of the Fortran shim
 * (wumingpic_gb300/fortran/wpic_shim2d.f90) -- and energy_history is computed on the host from
 * those arrays, as the driver computes it (2d/proj/weibel/app.f90:479-545).  Between the
 * diagnostic steps no particle or field array crosses the host link.
 *
 * Usage: wpic_driver2d <in.bin> <out.bin> nx ny np nsteps intvl_mom [precision]
 * precision: 0 = WPIC_FP64 (default), 2 = WPIC_MIXED (the same calls run the fused mixed step;
 * nx and ny multiples of 16).
 * in.bin: q[2], r[2] (doubles), then up(6, np, ny, 2), uf(6, nx+4, ny+4) (doubles),
 *         cumcnt(nx+1, ny, 2), np2(ny, 2) (int32), all in Fortran order.
 * out.bin: per diagnostic step: it (int32), up, np2, cumcnt, uf, mom(7, nx+2, ny+2, 2),
 *          energies (kinetic per species, E field, B field; doubles).
 * Grid: dx = 1, c dt/dx = 0.5, c = 1, gfac = 0.501, nxgs = nygs = 2, periodic.
 * Exit status 0 on success; a library status is printed with the call that returned it. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "wumingpic_gb300.h"

static int check(int st, const char* where) {
  if (st != WPIC_OK) fprintf(stderr, "wpic_driver2d: %s: status %d (%s)\n", where, st, wpic_status_string(st));
  return st;
}

#define CALL(expr)                         \
  do {                                     \
    if (check((expr), #expr)) return 2;    \
  } while (0)

static int read_all(FILE* f, void* p, size_t size, size_t n) { return fread(p, size, n, f) == n ? 0 : 1; }

/* energy_history's sums over the host arrays (2d/proj/weibel/app.f90:502-534) */
static void energy_history(const double* up, const int* np2, const double* uf, int nx, int ny, int np,
                           const double* r, double c, double* out) {
  const double pi = 4.0 * atan(1.0);
  for (int isp = 0; isp < 2; ++isp) {
    double v = 0.0;
    for (int j = 0; j < ny; ++j) {
      const double* row = up + ((size_t)isp * ny + j) * 6 * (size_t)np;
      for (int s = 0; s < np2[isp * ny + j]; ++s) {
        const double* u = row + 6 * (size_t)s;
        const double u2 = u[2] * u[2] + u[3] * u[3] + u[4] * u[4];
        v += r[isp] * (sqrt(1.0 + u2 / (c * c)) - 1.0);
      }
    }
    out[isp] = v;
  }
  double e = 0.0, b = 0.0;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const double* f = uf + 6 * ((size_t)(j + 2) * (nx + 4) + (i + 2));
      b += f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
      e += f[3] * f[3] + f[4] * f[4] + f[5] * f[5];
    }
  out[2] = e / (8.0 * pi);
  out[3] = b / (8.0 * pi);
}

int main(int argc, char** argv) {
  if (argc != 8 && argc != 9) {
    fprintf(stderr, "usage: %s in.bin out.bin nx ny np nsteps intvl_mom [precision]\n", argv[0]);
    return 1;
  }
  const int precision = argc == 9 ? atoi(argv[8]) : WPIC_FP64;
  const int nx = atoi(argv[3]), ny = atoi(argv[4]), np = atoi(argv[5]);
  const int nsteps = atoi(argv[6]), intvl = atoi(argv[7]);
  if (nx < 4 || ny < 4 || np < 1 || nsteps < 1 || intvl < 1) return 1;
  const size_t nup = (size_t)6 * np * ny * 2, nuf = (size_t)6 * (nx + 4) * (ny + 4);
  const size_t ncc = (size_t)(nx + 1) * ny * 2, nnp = (size_t)ny * 2, nmom = (size_t)7 * (nx + 2) * (ny + 2) * 2;
  double q[2], r[2];
  double* up = malloc(nup * sizeof(double));
  double* uf = malloc(nuf * sizeof(double));
  double* mom = malloc(nmom * sizeof(double));
  int* cumcnt = malloc(ncc * sizeof(int));
  int* np2 = malloc(nnp * sizeof(int));
  if (!up || !uf || !mom || !cumcnt || !np2) return 1;
  FILE* fi = fopen(argv[1], "rb");
  if (!fi) return 1;
  if (read_all(fi, q, sizeof(double), 2) || read_all(fi, r, sizeof(double), 2) ||
      read_all(fi, up, sizeof(double), nup) || read_all(fi, uf, sizeof(double), nuf) ||
      read_all(fi, cumcnt, sizeof(int), ncc) || read_all(fi, np2, sizeof(int), nnp)) {
    fclose(fi);
    return 1;
  }
  fclose(fi);
  FILE* fo = fopen(argv[2], "wb");
  if (!fo) return 1;

  /* particle__init, field__init, sort__init, bc__init (2d/proj/weibel/app.f90:330-346) */
  wpic_params prm = {0};
  prm.ndim = 6;
  prm.np = np;
  prm.nsp = 2;
  prm.nxgs = 2;
  prm.nxge = 2 + nx - 1;
  prm.nygs = 2;
  prm.nyge = 2 + ny - 1;
  prm.nys = prm.nygs;
  prm.nye = prm.nyge;
  prm.delx = 1.0;
  prm.delt = 0.5;
  prm.c = 1.0;
  prm.gfac = 0.501;
  prm.q[0] = q[0];
  prm.q[1] = q[1];
  prm.r[0] = r[0];
  prm.r[1] = r[1];
  prm.bc_kind = WPIC_BC_PERIODIC;
  prm.precision = precision;
  wpic_ctx* ctx = NULL;
  CALL(wpic_init_2d(&ctx, &prm, NULL));
  /* the initial state crosses once (the shim's upload at the first particle__solv) */
  CALL(wpic_put_particles(ctx, 0, up, np2, cumcnt));
  CALL(wpic_put_fields(ctx, uf));

  for (int it = 1; it <= nsteps; ++it) {
    /* 2d/proj/weibel/app.f90:101-106 */
    CALL(wpic_particle_solv(ctx));
    CALL(wpic_field_fdtd_i(ctx));
    CALL(wpic_bc_particle_x(ctx));
    CALL(wpic_bc_particle_y(ctx));
    CALL(wpic_sort_bucket(ctx));
    if (it % intvl) continue;
    /* 2d/proj/weibel/app.f90:119-125: the host arrays are refreshed on entry to mom_calc__accl */
    CALL(wpic_get_particles(ctx, 0, up, np2, cumcnt));
    CALL(wpic_get_fields(ctx, uf));
    CALL(wpic_mom_calc_accl(ctx));
    CALL(wpic_mom_calc_nvt(ctx, 1));
    CALL(wpic_bc_mom(ctx));
    CALL(wpic_get_mom(ctx, mom));
    double en[4];
    energy_history(up, np2, uf, nx, ny, np, r, prm.c, en);
    if (fwrite(&it, sizeof(int), 1, fo) != 1 || fwrite(up, sizeof(double), nup, fo) != nup ||
        fwrite(np2, sizeof(int), nnp, fo) != nnp || fwrite(cumcnt, sizeof(int), ncc, fo) != ncc ||
        fwrite(uf, sizeof(double), nuf, fo) != nuf || fwrite(mom, sizeof(double), nmom, fo) != nmom ||
        fwrite(en, sizeof(double), 4, fo) != 4) {
      fclose(fo);
      return 1;
    }
  }
  fclose(fo);
  CALL(wpic_finalize(ctx));
  free(up);
  free(uf);
  free(mom);
  free(cumcnt);
  free(np2);
  return 0;
}
