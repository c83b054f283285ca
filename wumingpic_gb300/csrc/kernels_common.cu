// Precision-independent 2D kernels: ghost fills and current folds (exact adds
// and copies), particle boundaries (round-toward-minus-infinity arithmetic as
// in the reference), particle migration between bucket rows, the bucket sort,
// gathers, layout conversions and the device-side synthetic loader.
#include <cstring>

#include "common.cuh"

namespace wpic {

// ---------------------------------------------------------------------------
// boundary_periodic__curre (2d/common/boundary_periodic.f90:357-508) with one
// rank: fold rows nys-2,nys-1 into nye-1,nye and nye+1,nye+2 into nys,nys+1,
// refresh the ghost rows, then (periodic x only) fold and refresh the ghost
// columns.  boundary_reconnection__curre has no x part
// (2d/proj/reconnection/boundary_reconnection.f90:364-502).
// Field rows: nys-2 -> 0, nys -> 2, nye -> ny+1, nye+2 -> ny+3 (same for x).
// ---------------------------------------------------------------------------
__global__ void k_curre_y(Dev2D d) {
  const Grid2D g = d.g;
  const int ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= g.nx + 4) return;
  const int ny = g.ny;
  for (int k = 0; k < 3; ++k) {
    double* u = d.uj + (size_t)k * g.fplane + ii;
    const size_t fp = g.fp;
    u[ny * fp] = u[ny * fp] + u[0];
    u[(ny + 1) * fp] = u[(ny + 1) * fp] + u[fp];
    u[2 * fp] = u[2 * fp] + u[(ny + 2) * fp];
    u[3 * fp] = u[3 * fp] + u[(ny + 3) * fp];
    u[(ny + 2) * fp] = u[2 * fp];
    u[(ny + 3) * fp] = u[3 * fp];
    u[0] = u[ny * fp];
    u[fp] = u[(ny + 1) * fp];
  }
}

__global__ void k_curre_x(Dev2D d) {
  const Grid2D g = d.g;
  const int jf = blockIdx.x * blockDim.x + threadIdx.x;
  if (jf >= g.ny + 4) return;
  const int nx = g.nx;
  for (int k = 0; k < 3; ++k) {
    double* u = d.uj + (size_t)k * g.fplane + (size_t)jf * g.fp;
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

void curre_fold2d(const Dev2D& d, cudaStream_t s) {
  k_curre_y<<<(d.g.nx + 4 + 127) / 128, 128, 0, s>>>(d);
  if (d.ph.bc == BC_PERIODIC) k_curre_x<<<(d.g.ny + 4 + 127) / 128, 128, 0, s>>>(d);
}

// ---------------------------------------------------------------------------
// boundary_periodic__mom (2d/common/boundary_periodic.f90:571-636, one rank: the y
// exchanges are self-exchanges) and boundary_reconnection__mom
// (2d/proj/reconnection/boundary_reconnection.f90:582-647, x ghosts folded onto the wall
// columns).  mom(7, nxgs-1:nxge+1, nys-1:nye+1, nsp); the x fold first over every row,
// then the y fold over every column, each thread doing its two statements in order.
// ---------------------------------------------------------------------------
__global__ void k_mom_fold_x(Dev2D d, double* mom) {
  const Grid2D g = d.g;
  const int nxm = g.nx + 2, nym = g.ny + 2;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;  // (l, jn, isp)
  if (t >= 7 * nym * d.ph.nsp) return;
  const int l = t % 7, r = t / 7;  // r = jn + nym * isp
  double* m = mom + (size_t)r * nxm * 7 + l;
  if (d.ph.bc != BC_PERIODIC) {  // walls: reconnection and shock
    m[7 * 1] = m[7 * 1] + m[0];
    m[7 * (size_t)g.nx] = m[7 * (size_t)g.nx] + m[7 * (size_t)(g.nx + 1)];
  } else {
    m[7 * 1] = m[7 * 1] + m[7 * (size_t)(g.nx + 1)];
    m[7 * (size_t)g.nx] = m[7 * (size_t)g.nx] + m[0];
  }
}

__global__ void k_mom_fold_y(Dev2D d, double* mom) {
  const Grid2D g = d.g;
  const int nxm = g.nx + 2, nym = g.ny + 2;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;  // (l, in) of one species
  const int isp = blockIdx.y;
  if (t >= 7 * nxm) return;
  const size_t col = 7 * (size_t)nxm;  // stride of one node row
  double* m = mom + (size_t)isp * nym * col + t;
  m[col * g.ny] = m[col * g.ny] + m[0];
  m[col] = m[col] + m[col * (g.ny + 1)];
}

void bc_mom2d(const Dev2D& d, double* mom, cudaStream_t s) {
  const int nx_threads = 7 * (d.g.ny + 2) * d.ph.nsp;
  k_mom_fold_x<<<(nx_threads + 255) / 256, 256, 0, s>>>(d, mom);
  k_mom_fold_y<<<dim3((7 * (d.g.nx + 2) + 255) / 256, d.ph.nsp), 256, 0, s>>>(d, mom);
}

// ---------------------------------------------------------------------------
// boundary_*__dfield (2d/common/boundary_periodic.f90:251-354;
// 2d/proj/reconnection/boundary_reconnection.f90:254-361): two-deep ghosts of df.
// ---------------------------------------------------------------------------
__global__ void k_dfield_y(Dev2D d) {
  const Grid2D g = d.g;
  const int ii = 2 + blockIdx.x * blockDim.x + threadIdx.x;  // interior columns nxs..nxe
  if (ii >= g.nx + 2) return;
  const int ny = g.ny;
  const size_t fp = g.fp;
  for (int k = 0; k < 6; ++k) {
    double* u = d.df + (size_t)k * g.fplane + ii;
    u[(ny + 2) * fp] = u[2 * fp];
    u[(ny + 3) * fp] = u[3 * fp];
    u[0] = u[ny * fp];
    u[fp] = u[(ny + 1) * fp];
  }
}

__global__ void k_dfield_x(Dev2D d) {
  const Grid2D g = d.g;
  const int jf = blockIdx.x * blockDim.x + threadIdx.x;
  if (jf >= g.ny + 4) return;
  const int nx = g.nx;
  double* u[6];
  for (int k = 0; k < 6; ++k) u[k] = d.df + (size_t)k * g.fplane + (size_t)jf * g.fp;
  if (d.ph.bc == BC_PERIODIC) {
    for (int k = 0; k < 6; ++k) u[k][0] = u[k][nx];
    for (int k = 0; k < 6; ++k) u[k][1] = u[k][nx + 1];
    for (int k = 0; k < 6; ++k) u[k][nx + 2] = u[k][2];
    for (int k = 0; k < 6; ++k) u[k][nx + 3] = u[k][3];
  } else {
    // window nxs..nxe = cells wx0..wx1: nxs-1 -> a, nxs -> a+1, nxs+1 -> a+2 (a = wx0 + 1);
    // nxe-1 -> e-1, nxe -> e, nxe+1 -> e+1 (e = wx1 + 2)
    const int a = g.wx0 + 1, e = g.wx1 + 2;
    u[0][a] = -u[0][a + 1];
    for (int k = 1; k <= 3; ++k) u[k][a] = u[k][a + 2];
    for (int k = 4; k <= 5; ++k) u[k][a] = -u[k][a + 1];
    if (d.ph.bc == BC_SHOCK) {  // boundary_shock__dfield (2d/proj/shock/boundary_shock.f90:397-405)
      for (int k = 0; k < 6; ++k) u[k][e + 1] = 0.0;
    } else {
      u[0][e] = -u[0][e - 1];
      for (int k = 1; k <= 3; ++k) u[k][e + 1] = u[k][e - 1];
      for (int k = 4; k <= 5; ++k) u[k][e] = -u[k][e - 1];
    }
  }
}

void dfield_ghost2d(const Dev2D& d, cudaStream_t s) {
  k_dfield_y<<<(d.g.nx + 127) / 128, 128, 0, s>>>(d);
  k_dfield_x<<<(d.g.ny + 4 + 127) / 128, 128, 0, s>>>(d);
}

// uf = uf + df over the whole ghosted extent (2d/common/field.f90:175-184)
__global__ void k_uf_add(Dev2D d) {
  const size_t n = (size_t)6 * d.g.fplane;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    d.uf[k] = d.uf[k] + d.df[k];
}
void uf_add2d(const Dev2D& d, cudaStream_t s) { k_uf_add<<<4 * 152, 256, 0, s>>>(d); }

// ---------------------------------------------------------------------------
// particle boundaries in x
//  periodic:     boundary_periodic__particle_x (2d/common/boundary_periodic.f90:61-96),
//                evaluated with round-toward-minus-infinity as the reference sets it (line 74)
//  reconnection: boundary_reconnection__particle_x (boundary_reconnection.f90:61-99),
//                reflection at x walls, all three momentum components reversed
// ---------------------------------------------------------------------------
// The periodic wrap: ipos = int(x/dx) rounded down is below nxgs exactly when x < nxgs dx and at
// or above nxge + 1 exactly when x >= (nxge + 1) dx (directed rounding is monotone and the bounds
// are integers).  A particle farther than 1e-12 of the domain's extent from both edges cannot
// wrap and is left alone without the FP64 division (GB300 runs FP64 at 1/64 of FP32); the others
// take the reference's arithmetic.
//
// The test itself uses no FP64 instruction: GB300 issues about two FP64 operations per clock per
// SM, so even compares and conversions of a double cost milliseconds over 5e8 particles.  For
// positive doubles the order of the IEEE bit patterns, read as 64-bit integers, is the order of
// the numbers, so the bounds are compared as integers (interior_bits); a bound that is not
// positive disables the shortcut (every particle then takes the exact path).
struct InteriorBits {
  long long lo, hi;  // a value v with lo < bits(v) < hi lies strictly inside the bounds
};

// lo < bits(v) < hi with 32-bit compares of the high and low words (the common case, a high
// word strictly between the bounds' high words, needs only the first test)
__device__ __forceinline__ bool inside_words(double v, const InteriorBits& b) {
  const int vh = __double2hiint(v);
  const int lh = (int)(b.lo >> 32), hh = (int)(b.hi >> 32);
  if (vh > lh && vh < hh) return true;
  const unsigned vl = (unsigned)__double2loint(v);
  const bool above = vh > lh || (vh == lh && vl > (unsigned)b.lo);
  const bool below = vh < hh || (vh == hh && vl < (unsigned)b.hi);
  return above && below;
}

__host__ __device__ inline InteriorBits interior_bits(double lo, double hi) {
  const double m = (fabs(lo) + fabs(hi)) * 1e-12;
  InteriorBits b;
  const double a = lo + m, c = hi - m;
  if (a > 0.0 && c > a) {
#ifdef __CUDA_ARCH__
    b.lo = __double_as_longlong(a);
    b.hi = __double_as_longlong(c);
#else
    memcpy(&b.lo, &a, 8);
    memcpy(&b.hi, &c, 8);
#endif
  } else {
    b.lo = 0x7fffffffffffffffLL;  // nothing is inside
    b.hi = 0;
  }
  return b;
}

__device__ __forceinline__ bool inside(double v, const InteriorBits& b) { return inside_words(v, b); }

// Row bounds k dx for k = j - 1 .. j + 2 as bit patterns, when every one of those products is an
// exact double (dx = 1, or any dx whose products with these integers do not round; checked with an
// FMA) and the lowest is not negative.  Then for a non-negative y, int(y/dx) rounded down equals
// j - 1, j or j + 1 exactly when the bits of y lie in [b[0], b[1]), [b[1], b[2]) or [b[2], b[3]),
// which integer compares of the 32-bit words decide without an FP64 instruction.
struct RowBounds {
  long long b[4];
  bool exact;
};

__device__ __forceinline__ RowBounds row_bounds(int j, double delx) {
  RowBounds r;
  r.exact = true;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const double kk = (double)(j - 1 + k);
    const double p = kk * delx;
    if (fma(kk, delx, -p) != 0.0 || p < 0.0) r.exact = false;
    r.b[k] = __double_as_longlong(p);
  }
  return r;
}

// a < b for the bit patterns of two non-negative doubles (a may be any double), by 32-bit words
__device__ __forceinline__ bool bits_less(double v, long long b) {
  const int vh = __double2hiint(v), bh = (int)(b >> 32);
  if (vh != bh) return vh < bh;
  return (unsigned)__double2loint(v) < (unsigned)b;
}

// jpos - j in {-1, 0, 1} from the exact bounds, or 2 when y lies outside [b[0], b[3])
__device__ __forceinline__ int row_step(double y, const RowBounds& r) {
  if (bits_less(y, r.b[1])) return bits_less(y, r.b[0]) ? 2 : -1;
  if (bits_less(y, r.b[2])) return 0;
  return bits_less(y, r.b[3]) ? 1 : 2;
}

InteriorBits x_interior(const Grid2D& g, double delx) {
  return interior_bits((double)g.nxgs * delx, (double)(g.nxgs + g.nx) * delx);
}

// The exact paths are separate, non-inlined functions: inlined, the compiler turns the rare branch
// into predicated FP64 instructions that every particle then pays for.
__device__ __noinline__ int floor_div_rd(double v, double delx) { return (int)__ddiv_rd(v, delx); }
__device__ __noinline__ int trunc_fp64(double v) { return (int)v; }

__device__ __forceinline__ double wrap_x_periodic(double x, const Grid2D& g, double delx, const InteriorBits& xin,
                                                  bool* changed) {
  const int nxge = g.nxgs + g.nx - 1;
  *changed = false;
  if (inside(x, xin)) return x;
  const int ipos = floor_div_rd(x, delx);
  const double L = __dmul_rd((double)g.nx, delx);
  if (ipos < g.nxgs) { *changed = true; return __dadd_rd(x, L); }
  if (ipos >= nxge + 1) { *changed = true; return __dsub_rd(x, L); }
  return x;
}

__global__ void k_particle_x(Dev2D d, Parts64 P, InteriorBits xin) {
  const int row = blockIdx.y;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= d.np2[row]) return;
  const size_t k = (size_t)row * d.cap + s;
  const Grid2D g = d.g;
  const double delx = d.ph.delx;
  double x = P.x[k];
  if (d.ph.bc == BC_PERIODIC) {
    bool changed;
    x = wrap_x_periodic(x, g, delx, xin, &changed);
    if (changed) P.x[k] = x;
  } else {
    const int nxs = g.nxgs + g.wx0, nxe = g.nxgs + g.wx1;  // the window; walls at nxs+1, nxe-1
    const int ipos = (int)(x / delx);
    bool flip = false;
    if (ipos < nxs + 1) {
      x = __dsub_rn(__dmul_rn((double)(2.0f * (float)(nxs + 1)), delx), x);
      flip = true;
    } else if (ipos >= nxe - 1) {
      x = __dsub_rn(__dmul_rn((double)(2.0f * (float)(nxe - 1)), delx), x);
      flip = true;
    }
    if (flip) {
      P.x[k] = x;
      P.ux[k] = -P.ux[k];
      P.uy[k] = -P.uy[k];
      P.uz[k] = -P.uz[k];
    }
  }
}

void particle_x2d(const Dev2D& d, const Parts64& P, cudaStream_t s) {
  dim3 grid((d.cap + 255) / 256, d.nrowjob);
  k_particle_x<<<grid, 256, 0, s>>>(d, P, x_interior(d.g, d.ph.delx));
}

// boundary_shock__injection (2d/proj/shock/boundary_shock.f90:255-297): reflection at the
// wall x = (nxs+1) dx with all momentum components reversed, and at the injection boundary
// xend = nxe dx + v0 dt (computed on the host, as the reference does, in FP64) with
// u_x -> 2 u0 - u_x; default rounding.
__global__ void k_injection(Dev2D d, Parts64 P, double u0, double xend) {
  const int row = blockIdx.y;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= d.np2[row]) return;
  const size_t k = (size_t)row * d.cap + s;
  const double delx = d.ph.delx;
  const int nxs = d.g.nxgs + d.g.wx0;
  const double x = P.x[k];
  const int ipos = (int)(x / delx);
  // products and differences rounded separately, as the reference evaluates them (no FMA)
  if (ipos < nxs + 1) {
    P.x[k] = __dsub_rn(__dmul_rn((double)(2.0f * (float)(nxs + 1)), delx), x);
    P.ux[k] = -P.ux[k];
    P.uy[k] = -P.uy[k];
    P.uz[k] = -P.uz[k];
  } else if (x > xend) {
    P.x[k] = __dsub_rn(__dmul_rn(2., xend), x);
    P.ux[k] = __dsub_rn(__dmul_rn(2., u0), P.ux[k]);
    P.uy[k] = -P.uy[k];
    P.uz[k] = -P.uz[k];
  }
}

void injection2d(const Dev2D& d, const Parts64& P, double u0, double xend, cudaStream_t s) {
  dim3 grid((d.cap + 255) / 256, d.nrowjob);
  k_injection<<<grid, 256, 0, s>>>(d, P, u0, xend);
}

// ---------------------------------------------------------------------------
// boundary_periodic__particle_y (2d/common/boundary_periodic.f90:99-248),
// first phase: classify every particle of a bucket row as staying, moving up
// (+y) or down (-y); wrap y with round-toward-minus-infinity as the reference
// does (line 124); record the up- and down-movers in slot order.  One CTA per
// (species, row).
// ---------------------------------------------------------------------------
constexpr int MIG_THREADS = 256;
constexpr int MIG_PER = 4;  // consecutive slots per thread in k_migrate_scan

// WRAPX: the periodic boundary_periodic__particle_x of the same particle first (the driver calls
// it right before particle_y), so that one pass over the row does both
template <bool WRAPX>
__global__ void __launch_bounds__(MIG_THREADS) k_migrate_scan(Dev2D d, Parts64 P, InteriorBits xin) {
  const Grid2D g = d.g;
  const int row = blockIdx.x;
  const int jj = row % g.ny;
  const int j = g.nygs + jj;
  const int nyge = g.nygs + g.ny - 1;
  const int n = d.np2[row];
  const size_t rb = (size_t)row * d.cap;
  const double delx = d.ph.delx;
  const double L = __dmul_rd((double)g.ny, delx);
  // jpos = int(y/dx) rounded down differs from j exactly when y < j dx or y >= (j + 1) dx; farther
  // than 1e-12 of the row's extent from both bounds the division is not needed
  const InteriorBits yin = interior_bits((double)j * delx, (double)(j + 1) * delx);
  const RowBounds yb = row_bounds(j, delx);
  // a chunk of MIG_THREADS * MIG_PER slots per iteration, slot c0 + q MIG_THREADS + thread
  // (coalesced loads, MIG_PER of them in flight per thread); the movers' list positions come from
  // the ballots of each sub-chunk q and the counts of the preceding warps (double-buffered: one
  // barrier per chunk)
  __shared__ int wu[2][MIG_PER][MIG_THREADS / 32], wd[2][MIG_PER][MIG_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lt = lanemask_lt();
  int base_u = 0, base_d = 0;  // movers of the chunks before (the same in every thread)
  int par = 0;
  for (int c0 = 0; c0 < n; c0 += MIG_THREADS * MIG_PER, par ^= 1) {
    int dir[MIG_PER];
    double y[MIG_PER];
#pragma unroll
    for (int q = 0; q < MIG_PER; ++q) {
      const int s = c0 + q * MIG_THREADS + threadIdx.x;
      y[q] = s < n ? P.y[rb + s] : 0.0;
    }
    if (WRAPX) {
      double x[MIG_PER];
#pragma unroll
      for (int q = 0; q < MIG_PER; ++q) {
        const int s = c0 + q * MIG_THREADS + threadIdx.x;
        x[q] = s < n ? P.x[rb + s] : 0.0;
      }
#pragma unroll
      for (int q = 0; q < MIG_PER; ++q) {
        const int s = c0 + q * MIG_THREADS + threadIdx.x;
        if (s >= n) continue;
        bool changed;
        const double xn = wrap_x_periodic(x[q], g, delx, xin, &changed);
        if (changed) P.x[rb + s] = xn;
      }
    }
    unsigned bu[MIG_PER], bd[MIG_PER];
#pragma unroll
    for (int q = 0; q < MIG_PER; ++q) {
      const int s = c0 + q * MIG_THREADS + threadIdx.x;
      dir[q] = 0;
      if (s < n) {
        int jpos = j;
        if (!inside(y[q], yin)) {
          const int st = yb.exact ? row_step(y[q], yb) : 2;
          jpos = st != 2 ? j + st : floor_div_rd(y[q], delx);
        }
        if (jpos != j) {
          if (jpos == j + 1) dir[q] = 1;
          else if (jpos == j - 1) dir[q] = 2;
          else atomicOr(d.err, EB_MOVED_TOO_FAR);
          if (dir[q] != 0) {
            double yn = y[q];
            if (jpos <= g.nygs - 1) yn = __dadd_rd(yn, L);
            else if (jpos >= nyge + 1) yn = __dsub_rd(yn, L);
            P.y[rb + s] = yn;
          }
        }
        d.mig[rb + s] = (int8_t)dir[q];
      }
      bu[q] = __ballot_sync(0xffffffffu, dir[q] == 1);
      bd[q] = __ballot_sync(0xffffffffu, dir[q] == 2);
      if (lane == 0) {
        wu[par][q][warp] = __popc(bu[q]);
        wd[par][q][warp] = __popc(bd[q]);
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < MIG_PER; ++q) {
      int ou = base_u + __popc(bu[q] & lt), od = base_d + __popc(bd[q] & lt);
#pragma unroll
      for (int w = 0; w < MIG_THREADS / 32; ++w) {
        const int a = wu[par][q][w], b = wd[par][q][w];
        if (w < warp) { ou += a; od += b; }
        base_u += a;
        base_d += b;
      }
      const int s = c0 + q * MIG_THREADS + threadIdx.x;
      if (dir[q] == 1) d.ulist[rb + ou] = s;
      if (dir[q] == 2) d.dlist[rb + od] = s;
    }
  }
  if (threadIdx.x == 0) {
    d.nup[row] = base_u;
    d.ndown[row] = base_d;
  }
}

void migrate_scan2d(const Dev2D& d, const Parts64& P, cudaStream_t s) {
  k_migrate_scan<false><<<d.nrowjob, MIG_THREADS, 0, s>>>(d, P, x_interior(d.g, d.ph.delx));
}

void wrapx_migrate_scan2d(const Dev2D& d, const Parts64& P, cudaStream_t s) {
  k_migrate_scan<true><<<d.nrowjob, MIG_THREADS, 0, s>>>(d, P, x_interior(d.g, d.ph.delx));
}

// ---------------------------------------------------------------------------
// Second phase of particle_y: the post-migration slot order of every row, in
// closed form.  The reference (boundary_periodic.f90:173-236, one rank, one
// thread) builds for each row an arrival buffer -- movers from the neighbouring
// rows in source order, then the ones wrapped through the periodic ghost row --
// and fills the row's holes in ascending slot order: first from the buffer;
// once the buffer is empty, from the tail of the row, taking the non-hole
// particles from the end downwards and dropping holes that the shrinking tail
// passes; leftover arrivals are appended.  Equivalently, with h holes, b
// arrivals and n particles:
//   b >= h : hole m <- arrival m ; slot n+k <- arrival h+k
//   b <  h : hole m (m < b) <- arrival m ; holes m >= b below n' = n-(h-b) <- the
//            non-hole slots of [n', n) in descending order ; the row ends at n'.
// One CTA of PW warps per (species, row) writes slist[t] = source slot of post-migration slot t:
// warp 0 lists the tail stayers (b < h), every warp counts the holes of its chunk of [0, nn), and
// with the counts of the chunks before it knows each hole's rank m; lanes take 4 consecutive slots.
// ---------------------------------------------------------------------------
constexpr int PW = 8;

__global__ void __launch_bounds__(PW * 32) k_migrate_plan(Dev2D d) {
  const Grid2D g = d.g;
  const int row = blockIdx.x;
  const int isp = row / g.ny, jj = row - isp * g.ny;
  const int rowS = isp * g.ny;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __shared__ int hcnt[PW];
  const size_t cap = d.cap;
  const int n = d.np2[row];
  const int h = d.nup[row] + d.ndown[row];
  int r1, r2, c1, c2;
  const int *l1, *l2;
  if (g.ny == 1) {
    r1 = row; l1 = d.dlist + r1 * cap; c1 = d.ndown[r1];
    r2 = row; l2 = d.ulist + r2 * cap; c2 = d.nup[r2];
  } else if (jj == 0) {
    r1 = row + 1; l1 = d.dlist + r1 * cap; c1 = d.ndown[r1];
    r2 = rowS + g.ny - 1; l2 = d.ulist + r2 * cap; c2 = d.nup[r2];
  } else if (jj == g.ny - 1) {
    r1 = row - 1; l1 = d.ulist + r1 * cap; c1 = d.nup[r1];
    r2 = rowS; l2 = d.dlist + r2 * cap; c2 = d.ndown[r2];
  } else {
    r1 = row - 1; l1 = d.ulist + r1 * cap; c1 = d.nup[r1];
    r2 = row + 1; l2 = d.dlist + r2 * cap; c2 = d.ndown[r2];
  }
  const int b = c1 + c2;
  int nn = n - h + b;
  if (nn > (int)cap) {
    if (threadIdx.x == 0) atomicOr(d.err, EB_CAPACITY);
    nn = (int)cap;
  }
  if (threadIdx.x == 0) d.np2new[row] = nn;
  const size_t rb = (size_t)row * cap;
  const unsigned lt = lanemask_lt();
  if (b < h && w == 0) {
    int k = 0;
    for (int t0 = n - 1; t0 >= nn; t0 -= 32) {
      const int t = t0 - lane;
      const bool st = t >= nn && d.mig[rb + t] == 0;
      const unsigned bal = __ballot_sync(0xffffffffu, st);
      if (st) d.tlist[rb + k + __popc(bal & lt)] = t;
      k += __popc(bal);
    }
  }
  constexpr int PER = 4 * 32;  // slots per warp iteration
  const int cs = ((nn + PW - 1) / PW + PER - 1) / PER * PER;
  const int lo = w * cs, hi = min(nn, lo + cs);
  auto is_hole = [&](int t) { return t < hi && t < n && d.mig[rb + t] != 0; };
  int cnt = 0;
  for (int t4 = lo + 4 * lane; t4 < hi; t4 += PER)
#pragma unroll
    for (int q = 0; q < 4; ++q) cnt += is_hole(t4 + q) ? 1 : 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if (lane == 0) hcnt[w] = cnt;
  __syncthreads();  // the chunk counts, and warp 0's tail list, are visible to every warp
  int m0 = 0;
  for (int q = 0; q < w; ++q) m0 += hcnt[q];
  for (int base = lo; base < hi; base += PER) {
    const int t4 = base + 4 * lane;
    bool hole[4];
    int c = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      hole[q] = is_hole(t4 + q);
      c += hole[q] ? 1 : 0;
    }
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    int m = m0 + incl - c;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int t = t4 + q;
      if (t >= hi) continue;
      int src = 0;
      int a = -1;  // arrival index
      if (t >= n) a = h + (t - n);
      else if (!hole[q]) src = (int)(rb + t);
      else if (m < b) a = m;
      else src = (int)(rb + d.tlist[rb + (m - b)]);
      if (hole[q]) ++m;
      if (a >= 0) src = a < c1 ? (int)((size_t)r1 * cap + l1[a]) : (int)((size_t)r2 * cap + l2[a - c1]);
      d.slist[rb + t] = src;
    }
    m0 += __shfl_sync(0xffffffffu, incl, 31);
  }
}

void migrate_plan2d(const Dev2D& d, cudaStream_t s) { k_migrate_plan<<<d.nrowjob, PW * 32, 0, s>>>(d); }

// ---------------------------------------------------------------------------
// sort__bucket (2d/common/sort.f90:36-82): stable counting sort of each row by
// the x cell i = int(x) (no division by delx, as in the reference).  One warp
// per (species, row): histogram in shared memory, exclusive scan -> cumcnt,
// then a rank pass in slot order where lanes with equal cells are ordered by
// __match_any_sync, which keeps the sort stable.  map[pos] = source slot.
// The input sequence is slist (post-migration order) or, if null, the row itself.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(32) k_sort_rank(Dev2D d, Parts64 P, const int* slist, const int* counts) {
  extern __shared__ int off[];
  const Grid2D g = d.g;
  const int row = blockIdx.x;
  const int lane = threadIdx.x;
  const int n = counts[row];
  const int nx = g.nx;
  const size_t rb = (size_t)row * d.cap;
  for (int k = lane; k <= nx; k += 32) off[k] = 0;
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
      atomicAdd(&off[cell], 1);
    }
  }
  __syncwarp();
  int* ccr = d.cc + (size_t)row * (nx + 1);
  int carry = 0;
  for (int k0 = 0; k0 < nx; k0 += 32) {
    const int k = k0 + lane;
    const int v = k < nx ? off[k] : 0;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const int excl = incl - v + carry;
    if (k < nx) {
      off[k] = excl;
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
    if (act) base = off[cell];
    __syncwarp();
    if (act && lane == __ffs(peers) - 1) off[cell] = base + __popc(peers);
    __syncwarp();
    if (act) d.map[rb + base + __popc(peers & lt)] = src;
  }
}

// The same stable counting sort with SW warps per row: warp w takes the w-th contiguous chunk of
// the input sequence.  Pass 1: per-warp cell histograms in shared memory (the cells kept in
// tlist); pass 2: per cell, the exclusive prefix over the warps plus the row's exclusive prefix
// over the cells (cumcnt); pass 3: every warp ranks its chunk in order from its own offsets, so
// the result is the single-warp sort's permutation.
constexpr int SW = 8;
constexpr int SORT_SMEM_MAX = 96 * 1024;

// int(x) (truncation) of a double by integer operations on its bits, for 0 <= x < 2^30; other
// values take the FP64 conversion.  Equal to (int)x wherever it answers.
__device__ __forceinline__ int trunc_double(double x) {
  const int hi = __double2hiint(x);
  const int e = ((hi >> 20) & 0x7ff) - 1023;
  if (hi >= 0 && e < 30) {
    if (e < 0) return 0;
    const unsigned mh = ((unsigned)hi & 0xfffffu) | 0x100000u;  // implicit bit + top 20 mantissa bits
    if (e <= 20) return (int)(mh >> (20 - e));
    const unsigned lo = (unsigned)__double2loint(x);
    return (int)((mh << (e - 20)) | (lo >> (52 - e)));
  }
  return trunc_fp64(x);
}

__global__ void __launch_bounds__(SW * 32) k_sort_rank_mw(Dev2D d, Parts64 P, const int* slist, const int* counts) {
  extern __shared__ int sh[];  // hist[SW][nx + 1], then tot[nx + 1]
  const Grid2D g = d.g;
  const int nx = g.nx, pitch = nx + 1;
  int* const tot = sh + SW * pitch;
  const int row = blockIdx.x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int n = counts[row];
  const size_t rb = (size_t)row * d.cap;
  for (int k = threadIdx.x; k < SW * pitch; k += SW * 32) sh[k] = 0;
  __syncthreads();
  const int chunk = ((n + SW - 1) / SW + 31) & ~31;
  const int t_lo = w * chunk, t_hi = min(n, t_lo + chunk);
  int* const hw = sh + w * pitch;
  for (int t = t_lo + lane; t < t_hi; t += 32) {
    const int src = slist ? slist[rb + t] : (int)(rb + t);
    int cell = trunc_double(P.x[src]) - g.nxgs;
    if (cell < 0 || cell >= nx) {
      atomicOr(d.err, EB_OUT_OF_RANGE);
      cell = cell < 0 ? 0 : nx - 1;
    }
    d.tlist[rb + t] = cell;
    atomicAdd(&hw[cell], 1);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < nx; k += SW * 32) {
    int acc = 0;
#pragma unroll
    for (int q = 0; q < SW; ++q) {
      const int v = sh[q * pitch + k];
      sh[q * pitch + k] = acc;
      acc += v;
    }
    tot[k] = acc;
  }
  __syncthreads();
  int* ccr = d.cc + (size_t)row * (nx + 1);
  if (w == 0) {
    int carry = 0;
    for (int k0 = 0; k0 < nx; k0 += 32) {
      const int k = k0 + lane;
      const int v = k < nx ? tot[k] : 0;
      int incl = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      if (k < nx) {
        tot[k] = incl - v + carry;
        ccr[k] = incl - v + carry;
      }
      carry += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0) ccr[nx] = carry;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < nx; k += SW * 32) {
    const int base = tot[k];
#pragma unroll
    for (int q = 0; q < SW; ++q) sh[q * pitch + k] += base;
  }
  __syncthreads();
  const unsigned lt = lanemask_lt();
  for (int t0 = t_lo; t0 < t_hi; t0 += 32) {
    const int t = t0 + lane;
    const bool act = t < t_hi;
    int src = 0, cell = -1 - lane;
    if (act) {
      src = slist ? slist[rb + t] : (int)(rb + t);
      cell = d.tlist[rb + t];
    }
    const unsigned peers = __match_any_sync(0xffffffffu, cell);
    int base = 0;
    if (act) base = hw[cell];
    __syncwarp();
    if (act && lane == __ffs(peers) - 1) hw[cell] = base + __popc(peers);
    __syncwarp();
    if (act) d.map[rb + base + __popc(peers & lt)] = src;
  }
}

void sort_rank2d(const Dev2D& d, const Parts64& P, const int* slist, cudaStream_t s) {
  const int* counts = slist ? d.np2new : d.np2;
  const size_t smem = (size_t)(SW + 1) * (d.g.nx + 1) * sizeof(int);
  if (smem <= (size_t)SORT_SMEM_MAX) {
    cudaFuncSetAttribute(k_sort_rank_mw, cudaFuncAttributeMaxDynamicSharedMemorySize, SORT_SMEM_MAX);
    k_sort_rank_mw<<<d.nrowjob, SW * 32, smem, s>>>(d, P, slist, counts);
  } else {
    k_sort_rank<<<d.nrowjob, 32, (d.g.nx + 1) * sizeof(int), s>>>(d, P, slist, counts);
  }
}

// dst[row][pos] = src[map[row][pos]] for pos < counts[row]
__global__ void k_gather(Dev2D d, Parts64 S, Parts64 D, const int* map, const int* counts) {
  const int row = blockIdx.y;
  const int pos = blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= counts[row]) return;
  const size_t k = (size_t)row * d.cap + pos;
  const size_t m = (size_t)map[k];
  D.x[k] = S.x[m];
  D.y[k] = S.y[m];
  D.ux[k] = S.ux[m];
  D.uy[k] = S.uy[m];
  D.uz[k] = S.uz[m];
  D.id[k] = S.id[m];
}

void gather2d(const Dev2D& d, const Parts64& src, const Parts64& dst, const int* map, const int* counts,
              cudaStream_t s) {
  dim3 grid((d.cap + 255) / 256, d.nrowjob);
  k_gather<<<grid, 256, 0, s>>>(d, src, dst, map, counts);
}

// ---------------------------------------------------------------------------
// layout conversions between the reference's particle layout up(ndim, np, ny, nsp)
// (AoS inside each row) and the device SoA; rows [row0, row0+nrows) of a staging block
// ---------------------------------------------------------------------------
__global__ void k_aos_to_soa(Dev2D d, const double* aos, int ndim, int np_host, int row0, Parts64 P) {
  const int row = row0 + blockIdx.y;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= d.np2[row]) return;
  const double* a = aos + ((size_t)blockIdx.y * np_host + s) * ndim;
  const size_t k = (size_t)row * d.cap + s;
  P.x[k] = a[0];
  P.y[k] = a[1];
  P.ux[k] = a[2];
  P.uy[k] = a[3];
  P.uz[k] = a[4];
  P.id[k] = ndim > 5 ? __double_as_longlong(a[5]) : 0;
}

__global__ void k_soa_to_aos(Dev2D d, double* aos, int ndim, int np_host, int row0, Parts64 P) {
  const int row = row0 + blockIdx.y;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= np_host) return;
  double* a = aos + ((size_t)blockIdx.y * np_host + s) * ndim;
  if (s >= d.np2[row] || s >= d.cap) {
    for (int c = 0; c < ndim; ++c) a[c] = 0.0;
    return;
  }
  const size_t k = (size_t)row * d.cap + s;
  a[0] = P.x[k];
  a[1] = P.y[k];
  a[2] = P.ux[k];
  a[3] = P.uy[k];
  a[4] = P.uz[k];
  if (ndim > 5) a[5] = __longlong_as_double(P.id[k]);
}

void aos_to_soa2d(const Dev2D& d, const double* aos, int ndim, int np_host, int row0, int nrows,
                  const Parts64& P, cudaStream_t s) {
  dim3 grid((np_host + 255) / 256, nrows);
  k_aos_to_soa<<<grid, 256, 0, s>>>(d, aos, ndim, np_host, row0, P);
}

void soa_to_aos2d(const Dev2D& d, double* aos, int ndim, int np_host, int row0, int nrows, const Parts64& P,
                  cudaStream_t s) {
  dim3 grid((np_host + 255) / 256, nrows);
  k_soa_to_aos<<<grid, 256, 0, s>>>(d, aos, ndim, np_host, row0, P);
}

__global__ void k_ref_to_soa(const double* ref, double* soa, int ncomp, int nslab) {
  const size_t n = (size_t)ncomp * nslab;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const size_t cell = k / ncomp, c = k - cell * ncomp;
    soa[c * nslab + cell] = ref[k];
  }
}
__global__ void k_soa_to_ref(const double* soa, double* ref, int ncomp, int nslab) {
  const size_t n = (size_t)ncomp * nslab;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const size_t cell = k / ncomp, c = k - cell * ncomp;
    ref[k] = soa[c * nslab + cell];
  }
}
void field_ref_to_soa(const double* ref, double* soa, int ncomp, int nslab, cudaStream_t s) {
  k_ref_to_soa<<<4 * 152, 256, 0, s>>>(ref, soa, ncomp, nslab);
}
void field_soa_to_ref(const double* soa, double* ref, int ncomp, int nslab, cudaStream_t s) {
  k_soa_to_ref<<<4 * 152, 256, 0, s>>>(soa, ref, ncomp, nslab);
}

// ---------------------------------------------------------------------------
// Device-side synthetic Weibel loader (same conventions as loader.py: species
// 0 = ions, 1 = electrons; co-located pairs; n0 = ppc per cell, uniform in the
// cell; electron beams +-drift alternating by particle; Philox4x32-10 streams).
// ---------------------------------------------------------------------------
__global__ void k_load_weibel2d(Dev2D d, int ppc, unsigned long long seed, double drift, int axis, double u_thi,
                                double u_the) {
  const Grid2D g = d.g;
  const int jj = blockIdx.y, isp = blockIdx.z;
  const int npr = g.nx * ppc;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int row = isp * g.ny + jj;
  if (k < npr && k < d.cap) {
    const uint2 key = make_uint2((unsigned)seed, (unsigned)(seed >> 32));
    const uint4 rp = philox4x32(make_uint4((unsigned)k, (unsigned)jj, 0u, 0u), key);
    const uint4 r1 = philox4x32(make_uint4((unsigned)k, (unsigned)jj, 1u + 2u * isp, 0u), key);
    const uint4 r2 = philox4x32(make_uint4((unsigned)k, (unsigned)jj, 2u + 2u * isp, 0u), key);
    const int cx = k / ppc;
    const size_t idx = (size_t)row * d.cap + k;
    d.A.x[idx] = ((double)(g.nxgs + cx) + (1.0 - u01(rp.x, rp.y))) * d.ph.delx;
    d.A.y[idx] = ((double)(g.nygs + jj) + (1.0 - u01(rp.z, rp.w))) * d.ph.delx;
    const double sd = isp == 0 ? u_thi : u_the;
    const double twopi = 6.283185307179586;
    const double a1 = u01(r1.x, r1.y), b1 = u01(r1.z, r1.w), a2 = u01(r2.x, r2.y), b2 = u01(r2.z, r2.w);
    double u[3];
    const double rad1 = sqrt(-2.0 * log(a1)), rad2 = sqrt(-2.0 * log(a2));
    u[0] = sd * rad1 * cos(twopi * b1);
    u[1] = sd * rad1 * sin(twopi * b1);
    u[2] = sd * rad2 * cos(twopi * b2);
    if (isp == 1 && drift != 0.0) u[axis] += (k % 2 == 0) ? drift : -drift;
    d.A.ux[idx] = u[0];
    d.A.uy[idx] = u[1];
    d.A.uz[idx] = u[2];
    d.A.id[idx] = -((long long)jj * npr + k + 1);
  }
  if (k <= g.nx && blockIdx.x == 0) {
    for (int kk = threadIdx.x; kk <= g.nx; kk += blockDim.x) d.cc[(size_t)row * (g.nx + 1) + kk] = kk * ppc;
  }
  if (k == 0) d.np2[row] = npr < d.cap ? npr : d.cap;
}

void load_weibel2d_ppc(const Dev2D& d, int ppc, unsigned long long seed, double drift, int drift_axis,
                       double u_thi, double u_the, cudaStream_t s) {
  dim3 grid((d.g.nx * ppc + 255) / 256, d.g.ny, d.ph.nsp);
  k_load_weibel2d<<<grid, 256, 0, s>>>(d, ppc, seed, drift, drift_axis, u_thi, u_the);
}

}  // namespace wpic
