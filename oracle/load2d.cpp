// load2d.cpp -- seeded 2D Weibel plasma written straight into the reference layout
// (TEST AND BENCHMARK INFRASTRUCTURE).
//
// Used only by bench.py's reference arm, which times the oracle's step on the full
// benchmark grid: the numpy loader (wumingpic_gb300/loader.py) needs minutes and
// several times the state's memory for 5e8 particles; this one fills the arrays
// row-parallel in place.  The state has the numpy loader's shape and distribution --
// ions and electrons co-located, uniform in each cell, cell-major inside each row,
// isotropic Gaussian momenta (four-velocity) with +-drift alternating on the
// electrons, ids -pid bit-cast into the last real(8) slot, bucket-sorted cumcnt
// (2d/proj/weibel/app.f90:405-431, 468; 2d/common/sort.f90:64-69) -- but its random
// numbers come from a counter hash (splitmix64 of seed, row, particle, draw), not from
// numpy's Philox, so the two loaders give different plasmas of the same configuration.
#include <cmath>
#include <cstdint>
#include <cstring>

namespace {

inline uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ULL;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

// uniform in [0, 1) from the top 53 bits of a hash of (seed, a, b, draw)
inline double unif(uint64_t seed, uint64_t a, uint64_t b, uint64_t draw) {
  const uint64_t h = mix64(mix64(mix64(seed ^ (a * 0x100000001b3ULL)) ^ b) + draw);
  return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

}  // namespace

extern "C" {

// up(ndim=6, np, ny, nsp), cumcnt(nx+1, ny, nsp), np2(ny, nsp), Fortran order; uf is left to
// the caller (zero fields).  sd[isp] is the thermal spread of species isp; the electrons
// (species nsp-1) carry +-drift along drift_axis (0, 1, 2 = x, y, z).  Returns 0, or 2 if a
// row's ppc * nx particles do not fit np.
int orc2d_load_weibel(double* up, int* cumcnt, int* np2, int nx, int ny, int np, int nsp, int ppc, int nxgs,
                      int nygs, double delx, const double* sd, double drift, int drift_axis, unsigned long long seed) {
  const long long npr = (long long)nx * ppc;
  if (npr > np) return 2;
  const int ndim = 6;
  const double two_pi = 8.0 * std::atan(1.0);
#pragma omp parallel for schedule(static)
  for (int j = 0; j < ny; ++j) {
    for (int isp = 0; isp < nsp; ++isp) {
      double* row = up + ((size_t)isp * ny + j) * (size_t)ndim * np;
      for (long long k = 0; k < npr; ++k) {
        double* p = row + (size_t)k * ndim;
        // positions shared by the species (zero initial charge density)
        p[0] = (nxgs + (double)(k / ppc) + unif(seed, j, k, 0)) * delx;
        p[1] = (nygs + (double)j + unif(seed, j, k, 1)) * delx;
        for (int a = 0; a < 3; a += 2) {
          // two normals per Box-Muller pair; the third component takes the first of a second pair
          const double r1 = 1.0 - unif(seed, j, k, 2 + 8 * isp + a), r2 = unif(seed, j, k, 3 + 8 * isp + a);
          const double rad = std::sqrt(-2.0 * std::log(r1));
          p[2 + a] = sd[isp] * rad * std::cos(two_pi * r2);
          if (a == 0) p[3] = sd[isp] * rad * std::sin(two_pi * r2);
        }
        if (isp == nsp - 1 && drift != 0.0) p[2 + drift_axis] += (k % 2 == 0) ? drift : -drift;
        const long long pid = -((long long)j * npr + k + 1);
        std::memcpy(&p[5], &pid, sizeof pid);
      }
      np2[(size_t)isp * ny + j] = (int)npr;
      int* cc = cumcnt + ((size_t)isp * ny + j) * (nx + 1);
      for (int i = 0; i <= nx; ++i) cc[i] = i * ppc;
    }
  }
  return 0;
}

}  // extern "C"
