// Internal declarations shared by the C-ABI unit (capi.cu) and the kernel units.
//
// Device data layout (2D; one GPU holds the whole domain):
//   fields   SoA, component-major, with the reference's +-2 ghost layers:
//            F[c][jj][ii], jj = j-(nys-2) in [0,ny+4), ii = i-(nxgs-2) in [0,nx+4)
//   particles SoA per species and row ("bucket row" = the reference's storage row j),
//            slot s of row jj of species isp at ((isp*ny)+jj)*cap + s; inside a row the
//            particles are bucket-sorted by x cell, cumcnt giving the cell offsets
//   cumcnt   [isp][jj][0..nx]  (cumcnt(nxgs+ii, j, isp))
//   np2      [isp][jj]
#pragma once
#include <cmath>
#include <cuda_runtime.h>
#include <cstdint>

namespace wpic {

enum Status : int {
  ST_OK = 0,
  ST_CG_NOT_CONVERGED = 1,
  ST_CAPACITY = 2,
  ST_OUT_OF_RANGE = 3,
  ST_MOVED_TOO_FAR = 4,
  ST_NONFINITE = 5,
  ST_BAD_ARGUMENT = 6,
  ST_CUDA = 7,
  ST_NOT_INITIALISED = 8,
};

// device error word bits
enum ErrBit : int {
  EB_CAPACITY = 1,
  EB_OUT_OF_RANGE = 2,
  EB_MOVED_TOO_FAR = 4,
  EB_CG = 8,
  // a bulk (TMA) copy into shared memory did not complete within the kernel's wait limit;
  // the copy may still be in flight when the CTA returns, so the context is finished
  EB_STAGING_TIMEOUT = 16,
};

enum Bc : int { BC_PERIODIC = 0, BC_RECONNECTION = 1, BC_SHOCK = 2 };

// modes of the particle push kernels: particle__solv, particle__solv_vay, mom_calc__accl
enum PushMode : int { PUSH_BORIS = 0, PUSH_VAY = 1, PUSH_MOM = 2 };

struct Grid2D {
  int nx, ny;       // interior cells
  int nxgs, nygs;   // reference index of the first interior cell (nxgs, nys)
  int fp;           // field row pitch = nx + 4
  int fplane;       // (nx + 4) * (ny + 4)
  int ncell;        // nx * ny
  int wx0, wx1;     // active x window nxs..nxe as interior cell indices (all cells unless set)
};

struct Phys {
  double delx, delt, c, gfac;
  double q[2], r[2];
  double p_d_delx;  // particle__init:  1./delx        (2d/common/particle.f90:41)
  double d_delx;    // field__init:     1./delx        (2d/common/field.f90:58)
  double d_delt;    // field__init:     1./delt        (2d/common/field.f90:59)
  double f1, f2, f3, f4, f5, pi;
  int nsp;
  int bc;
};

struct Parts64 {
  double *x, *y, *ux, *uy, *uz;
  long long* id;
};

// ---- mixed-precision particle storage (2D) ----
// Particles live in bins of one 16 x 16-cell tile and one species, bin = tile * nsp + isp,
// tile = ty * ntx + tx.  Inside a bin every cell owns a column of bdep[bin] slots:
// slot (k, c) for cell c = ly * 16 + lx lies in layer boff[bin] + k, so the cell of a particle
// is implicit.  Position = that cell plus an FP32 offset in [0, 1) per dimension; momenta FP32;
// 64-bit id.  Each 256-slot layer holds the slots of the tile's cells in order, a slot being the
// particle's 8 words (below), so a warp's 32 cells are 1 KB of contiguous memory.
// A push compacts each column in place (stayers to the bottom) and writes the particles that
// change cell to the top of their new cell's column, from slot bdep - 1 downwards; the arrival
// kernel then moves them, in key order, to just above the stayers.  The depth of a bin grows
// (the host re-lays out the bins) when its columns come close to full.
constexpr int MIX_TS = 16;
constexpr int MIX_TC = MIX_TS * MIX_TS;
constexpr int MIX_FLUSH = 64;  // particles a push thread sums in registers between fixed-point flushes
constexpr int MIX_MAX_DEPTH = 32767;  // slot indices fit the 16-bit field of the arrival key
// A slot is 8 consecutive 32-bit words (32 bytes): ox, oy, ux, uy, uz, id low, id high, arrival key.
// Slot (k, c) of a bin lies at word ((boff + k) * 256 + c) * 8, so a warp reading slot k of 32
// neighbouring cells reads 1 KB contiguously, and a thread moves a particle with two 16-byte
// accesses.
constexpr int MIX_W = 8;             // 32-bit words per slot
constexpr int MIX_OX = 0, MIX_OY = 1, MIX_UX = 2, MIX_UY = 3, MIX_UZ = 4;
constexpr int MIX_IDLO = 5, MIX_IDHI = 6, MIX_KEY = 7;
constexpr int MIX_PL = MIX_W * MIX_TC;  // 32-bit words per layer

struct Mix2D {
  // fixed-point current accumulation of the push: v = hi / s1 + lo / s2 with int32 hi, lo
  float fx_s1, fx_s2, fx_is1f;
  double fx_is1, fx_is2;
  // FP32 constants of the push and deposit, rounded once from the FP64 parameters:
  // per species q/r dt/2, q dt/r, q dx/dt, q; then dt/dx, c, 1/c^2
  float k_fac1[2], k_fac2[2], k_qdd[2], k_q[2];
  float k_dtdx, k_c, k_ic2;
  int k_xend_cell;     // shock: the injection end in cells from nxgs as an integer cell and an FP32
  float k_xend_frac;   // fraction in [0, 1), and u0 (set every step)
  float k_u0;
  int ntx, nty, ntile, nbin;
  float* P;            // particle layers, MIX_PL words each
  long long* boff;     // [nbin] first layer of each bin
  int* bdep;           // [nbin] slots per cell column of each bin
  int* cnt;            // [nbin][256] particles per column (the push's input count)
  int* ccnt;           // [nbin][256] stayers after the push's compaction
  int* acnt;           // [nbin][256] arrivals written by the push (zero between steps)
  int* bneed;          // [nbin] largest count + 2 x arrivals over a bin's columns in the last step
  int* grow;           // nonzero when some bin's need passed 7/8 of its depth
  unsigned long long* ujx;  // [3][ny+4][nx+4] current in fixed point (units 1/fx_s2), summed exactly
};

// first word of slot (k, c) of bin `bin`; the components at + MIX_OX ... + MIX_KEY
__device__ inline float* mix_slot(const Mix2D& m, int bin, int k, int c) {
  return m.P + (((size_t)m.boff[bin] + k) * MIX_TC + c) * MIX_W;
}

struct CGState {
  double sum_g, eps, sumr_g, sum2_g, sum1_g, av, bv;
  int ite, active, fixed, pad;
};

struct Dev2D {
  Grid2D g;
  Phys ph;
  int cap;          // device slots per row per species
  int nrowjob;      // nsp * ny
  Parts64 A, B, C;  // A = "up" (sorted state), B = "gp" (scratch / new state), C = migration staging
  int* cc;          // cumcnt [nsp][ny][nx+1]
  int* np2;         // [nsp][ny]
  double *uf, *df, *uj;  // [6|6|3][ny+4][nx+4]
  double* gkl;           // [3][ny][nx]
  double* cellJ;         // [75][ny][nx]  per-cell 5x5 current tiles (3 components)
  double *phi, *p, *r, *ap, *b;  // [3][ny][nx]
  double* partials;      // reduction partials
  int nred;              // number of reduction blocks per component
  CGState* cg;           // [3]
  int ite_max;
  double cg_rtol;        // CG stopping tolerance relative to ||b|| (the reference's 1e-6)
  // migration / sort scratch
  int8_t* mig;           // per slot: 0 stay, 1 up (+y), 2 down (-y)
  int *ulist, *dlist, *tlist, *slist, *map;  // per slot
  int *nup, *ndown, *np2new;                 // per row job
  int* err;              // device error word
  double* red_out;       // misc reduction output (energy)
  int mixed;             // 1: particles in the mixed-precision bins below
  Mix2D m;
};

// ---- launchers: precision-dependent kernels exist in two builds ----
#define WPIC_DECLARE_FP_LAUNCHERS                                                          \
  void push2d(const Dev2D& d, cudaStream_t s);                                             \
  void push_vay2d(const Dev2D& d, cudaStream_t s);                                         \
  void mom_accl2d(const Dev2D& d, cudaStream_t s);                                         \
  void mom_nvt2d(const Dev2D& d, const Parts64& P, double* mom, cudaStream_t s);           \
  void deposit2d(const Dev2D& d, cudaStream_t s);                                          \
  void gkl2d(const Dev2D& d, cudaStream_t s);                                              \
  void cg_init2d(const Dev2D& d, cudaStream_t s);                                          \
  void cg_iter_ap2d(const Dev2D& d, cudaStream_t s);                                       \
  void cg_iter_update2d(const Dev2D& d, cudaStream_t s);                                   \
  void cg_iter_p2d(const Dev2D& d, cudaStream_t s);                                        \
  void cg_store2d(const Dev2D& d, cudaStream_t s);                                         \
  void efield2d(const Dev2D& d, cudaStream_t s);                                           \
  void energy2d(const Dev2D& d, cudaStream_t s);                                           \
  void energy_fields_fin2d(const Dev2D& d, cudaStream_t s);

namespace exact { WPIC_DECLARE_FP_LAUNCHERS }
namespace fast { WPIC_DECLARE_FP_LAUNCHERS }

// ---- precision-independent kernels (integer work, copies, exact adds) ----
void curre_fold2d(const Dev2D& d, cudaStream_t s);
void bc_mom2d(const Dev2D& d, double* mom, cudaStream_t s);
void mix_moments2d(const Dev2D& d, double* mom, cudaStream_t s);
void dfield_ghost2d(const Dev2D& d, cudaStream_t s);
void uf_add2d(const Dev2D& d, cudaStream_t s);
void particle_x2d(const Dev2D& d, const Parts64& P, cudaStream_t s);
void injection2d(const Dev2D& d, const Parts64& P, double u0, double xend, cudaStream_t s);
// adjoint of the FP64 2D step (adjoint2d.cu); f32 (6 field planes of FP32 scratch, or null):
// the per-particle sweeps in FP32
void adj_field(const Dev2D& d, double* luf, double* ldf, double* luj, cudaStream_t s);
void adj_field_after_cg(const Dev2D& d, double* luf, double* lg, double* luj, cudaStream_t s);
void adj_unsort(const Dev2D& d, const Parts64& lA, const Parts64& lB, cudaStream_t s);
void adj_particles(const Dev2D& d, const double* luj, const Parts64& lA, const Parts64& lB, double* tmp,
                   double* ltmp, double* luf, float* f32, cudaStream_t s);
void adj_fill_rand(double* v, size_t n, unsigned seed, cudaStream_t s);
void adj_field_fold_T(const Dev2D& d, double* luj, cudaStream_t s);
void adj_field_ghost_T(const Dev2D& d, double* ldf, cudaStream_t s);
void adj_field_efield_T(const Dev2D& d, double* ldf, double* luf, double* luj, cudaStream_t s);
void adj_field_gkl_T(const Dev2D& d, const double* lg, double* luf, double* luj, cudaStream_t s);
void adj_field_tmp(const Dev2D& d, double* tmp, cudaStream_t s);
void adj_field_tmp_T(const Dev2D& d, const double* ltmp, double* luf, cudaStream_t s);
void adj_keep_interior(const Dev2D& d, double* v, int ncomp, cudaStream_t s);
void adj_axpy(double* dst, const double* x, const double* v, double h, size_t n, cudaStream_t s);
void adj_dot_parts(const Dev2D& d, const Parts64& L, const Parts64& P, double scale, double* out, cudaStream_t s);
void adj_deposit_only(const Dev2D& d, const double* luj, const Parts64& lA, const Parts64& lB, float* f32,
                      cudaStream_t s);
void adj_push_fields(const Dev2D& d, const Parts64& lB, const Parts64& lA, double* tmp, double* ltmp, double* luf,
                     float* f32, cudaStream_t s);
void adj_dot(const double* a, const double* b, size_t n, double* out, cudaStream_t s);
void migrate_scan2d(const Dev2D& d, const Parts64& P, cudaStream_t s);
// boundary_periodic__particle_x and the first phase of particle_y in one pass (periodic runs)
void wrapx_migrate_scan2d(const Dev2D& d, const Parts64& P, cudaStream_t s);
void migrate_plan2d(const Dev2D& d, cudaStream_t s);
void sort_rank2d(const Dev2D& d, const Parts64& P, const int* slist, cudaStream_t s);
void gather2d(const Dev2D& d, const Parts64& src, const Parts64& dst, const int* map, const int* counts,
              cudaStream_t s);
void aos_to_soa2d(const Dev2D& d, const double* aos, int ndim, int np_host, int row0, int nrows,
                  const Parts64& P, cudaStream_t s);
void soa_to_aos2d(const Dev2D& d, double* aos, int ndim, int np_host, int row0, int nrows, const Parts64& P,
                  cudaStream_t s);
void field_ref_to_soa(const double* ref, double* soa, int ncomp, int nslab, cudaStream_t s);
void field_soa_to_ref(const double* soa, double* ref, int ncomp, int nslab, cudaStream_t s);
// ---- mixed-precision path (mixed2d.cu) ----
int mix_setup2d(const Dev2D& d, void* tmap_out);  // CUtensorMap of uf for the TMA tile loads; kernel attributes
// copy every column of the layout `from` (P, boff, bdep) into the layout of d.m (counts unchanged)
void mix_relayout2d(const Dev2D& d, const float* from_P, const long long* from_boff, cudaStream_t s);
// initial slots per column for a column of n particles (with the room the first pushes need)
int mix_initial_depth(double n, double c_dt_dx);
void mix_push_deposit2d(const Dev2D& d, const void* tmap, bool vay, cudaStream_t s);
void mix_curre_refresh2d(const Dev2D& d, cudaStream_t s);
void mix_migrate2d(const Dev2D& d, cudaStream_t s);
void mix_put2d(const Dev2D& d, const double* aos, int ndim, int np_host, int isp, int ty0, int nty, cudaStream_t s);
void mix_binmax2d(const Dev2D& d, cudaStream_t s);  // bneed[bin] = largest cell count in d.cc
void mix_count_rows2d(const Dev2D& d, cudaStream_t s);  // cumcnt and np2 of the reference layout
void mix_get2d(const Dev2D& d, double* aos, int ndim, int np_host, int isp, int ty0, int nty, cudaStream_t s);
void mix_load_weibel2d(const Dev2D& d, int ppc, unsigned long long seed, double drift, int drift_axis,
                       double u_thi, double u_the, cudaStream_t s);
void mix_energy2d(const Dev2D& d, cudaStream_t s);

void load_weibel2d_ppc(const Dev2D& d, int ppc, unsigned long long seed, double drift, int drift_axis,
                       double u_thi, double u_the, cudaStream_t s);

// ---- 3D FP64 path ----
// boundary_shock__injection's right end, xend = nxe dx + v0 dt with v0 = u0 / sqrt(1 + u0^2/c^2)
// (2d/proj/shock/boundary_shock.f90, 3d/proj/shock/boundary_shock.f90:437): every product and
// sum rounded on its own, as the reference evaluates it (no contraction into an FMA)
inline double shock_xend_value(int nxe, double delx, double u0, double c, double delt) {
  volatile double a = nxe * delx;
  volatile double v0 = u0 / std::sqrt(1 + (u0 * u0) / (c * c));
  volatile double b = v0 * delt;
  return a + b;
}

struct Grid3D {
  int nx, ny, nz;
  int nxgs, nygs, nzgs;
  int wx0, wx1;    // the active x window nxs..nxe as local cells (0, nx - 1 unless a shock run)
  int fp;          // nx + 4: row pitch of a ghosted field
  size_t fplane;   // (nx + 4)(ny + 4)
  size_t fvol;     // (nx + 4)(ny + 4)(nz + 4): one component of a ghosted field
  size_t ncell;    // nx ny nz
};

struct Parts3D {
  double *x, *y, *z, *ux, *uy, *uz;
  long long* id;
};

// ---- mixed-precision particle storage (3D) ----
// The 2D scheme in three dimensions: bins of one 8 x 8 x 4-cell tile and one species,
// bin = tile * nsp + isp, tile = (tz * nty + ty) * ntx + tx.  Inside a bin every cell
// c = (lz * 8 + ly) * 8 + lx owns a column of bdep[bin] slots; slot (k, c) lies in layer
// boff[bin] + k.  Position = the column's cell plus three FP32 offsets in [0, 1); momenta FP32;
// 64-bit id: a slot is 8 consecutive 32-bit words (ox, oy, oz, ux, uy, uz, id low word, id high
// word), 32 bytes, the layer's 256 slots in cell order; the arrival key of a slot lies in a
// separate array of one 32-bit word per slot.  The push compacts each column in place and
// writes the particles that change cell to the top of their new column; the arrival kernel moves
// them, in key order, to just above the stayers; bins grow when their columns come close to full.
constexpr int M3_TX = 8, M3_TY = 8, M3_TZ = 4;
constexpr int M3_TC = M3_TX * M3_TY * M3_TZ;  // cells per tile = threads of the tile kernels
constexpr int M3_W = 8;  // 32-bit words per slot
constexpr int M3_OX = 0, M3_OY = 1, M3_OZ = 2, M3_UX = 3, M3_UY = 4, M3_UZ = 5, M3_IDLO = 6, M3_IDHI = 7;
constexpr int M3_PL = M3_W * M3_TC;  // 32-bit words per layer

struct Mix3D {
  // fixed-point current: v = hi / s1 + lo / s2 (int32 planes in shared memory), global sums in
  // units of 1 / s2 (int64)
  float fx_s1, fx_s2, fx_is1f;
  double fx_is2;
  int ntx, nty, ntz, ntile, nbin;
  float* P;            // particle layers, M3_PL words each
  int* K;              // arrival keys, one per slot (M3_TC per layer)
  long long* boff;     // [nbin] first layer of each bin
  int* bdep;           // [nbin] slots per cell column
  int* cnt;            // [nbin][256] particles per column (the push's input count)
  int* ccnt;           // [nbin][256] stayers after the push's compaction
  int* acnt;           // [nbin][256] arrivals written by the push (zero between steps)
  int* bneed;          // [nbin] largest count + 2 x arrivals over a bin's columns in the last step
  int* grow;           // nonzero when some bin's need passed 7/8 of its depth
  unsigned long long* ujx;  // [3][fvol] current in fixed point (units 1/fx_s2), summed exactly
};

__device__ inline float* mix3_slot(const Mix3D& m, int bin, int k, int c) {
  return m.P + (((size_t)m.boff[bin] + k) * M3_TC + c) * M3_W;
}
__device__ inline int* mix3_key(const Mix3D& m, int bin, int k, int c) {
  return m.K + ((size_t)m.boff[bin] + k) * M3_TC + c;
}

struct Dev3D {
  Grid3D g;
  Phys ph;
  int cap;          // device slots per row (j, k) per species
  int nrow;         // nsp * nz * ny; row = (isp * nz + kk) * ny + jj, the reference's (j, k) loop order
  Parts3D A, B;     // A = "up" (sorted state), B = "gp" (new state)
  int* cc;          // cumcnt [row][nx+1]
  int *np2, *np2new;
  double *uf, *df, *uj;          // [6|6|3][nz+4][ny+4][nx+4]
  double* gkl;                   // [3][nz][ny][nx]
  double* cellJ;                 // [cell][375]: per-cell 5x5x5 current stencils (3 components)
  double *phi, *p, *r, *ap, *b;  // [3][nz][ny][nx]
  double* partials;
  int nred;
  CGState* cg;
  int ite_max;
  // migration / sort scratch
  int8_t* mig;      // per slot: 0 stay, else 1 + direction code (dz + 1) * 3 + (dy + 1)
  int* glist;       // per row: movers grouped by direction group (0..7), slot order inside a group
  int *gcnt, *goff; // [row][8]: movers per direction group and their offset in glist
  int *tlist, *slist, *map;
  int* err;
  double* red_out;
  Mix3D m;          // the mixed path's particle bins (the FP64 particle arrays are then unused)
};

#define WPIC_DECLARE_FP3_LAUNCHERS                       \
  void push3d(const Dev3D& d, cudaStream_t s);           \
  void push_vay3d(const Dev3D& d, cudaStream_t s);       \
  void mom_accl3d(const Dev3D& d, cudaStream_t s);       \
  void mom_nvt3d(const Dev3D& d, const Parts3D& P, double* mom, cudaStream_t s); \
  void deposit3d(const Dev3D& d, cudaStream_t s);        \
  void gkl3d(const Dev3D& d, cudaStream_t s);            \
  void cg_init3d(const Dev3D& d, cudaStream_t s);        \
  void cg_iter_ap3d(const Dev3D& d, cudaStream_t s);     \
  void cg_iter_update3d(const Dev3D& d, cudaStream_t s); \
  void cg_iter_p3d(const Dev3D& d, cudaStream_t s);      \
  void cg_store3d(const Dev3D& d, cudaStream_t s);       \
  void efield3d(const Dev3D& d, cudaStream_t s);         \
  void energy3d(const Dev3D& d, cudaStream_t s);          \
  void energy_fields_fin3d(const Dev3D& d, cudaStream_t s);

namespace exact { WPIC_DECLARE_FP3_LAUNCHERS }
namespace fast { WPIC_DECLARE_FP3_LAUNCHERS }

// mixed-precision 3D: FP32 constants rounded once on the host; the shock's injection end split
// into an integer cell and an FP32 fraction (cells from nxgs), and u0 (set every step)
struct Mix3Const {
  float fac1[2], fac2[2], qdd[2];
  float dtdx, c, ic2;
  int xend_cell;
  float xend_frac, u0;
};
bool mix3_shape_ok(int nx, int ny, int nz);
// CUtensorMap of uf for the tile loads, kernel attributes; 0 on success
int mix3_setup(const Dev3D& d, void* tmap_out);
// the fused FP32 push + deposit + column compaction (ujx cleared first)
void mix3_push(const Dev3D& d, const Mix3Const& k, const void* tmap, bool vay, cudaStream_t s);
void mix3_arrive(const Dev3D& d, cudaStream_t s);
void mix3_fix(const Dev3D& d, cudaStream_t s);  // uj = ujx / s2 over the ghosted extent
void mix3_relayout(const Dev3D& d, const float* from_P, const long long* from_boff, cudaStream_t s);
int mix3_initial_depth(double n, double c_dt_dx);
void mix3_binmax(const Dev3D& d, cudaStream_t s);        // bneed[bin] = largest cell count in d.cc
void mix3_count_rows(const Dev3D& d, cudaStream_t s);    // cumcnt and np2 of the reference layout
// reference layout <-> bins for the rows of species isp and z layers 4 tz .. 4 tz + 3 (aos holds
// those 4 ny rows, np_host slots each)
void mix3_put(const Dev3D& d, const double* aos, int ndim, int np_host, int isp, int tz, cudaStream_t s);
void mix3_get(const Dev3D& d, double* aos, int ndim, int np_host, int isp, int tz, cudaStream_t s);
void mix3_load_weibel(const Dev3D& d, int ppc, unsigned long long seed, double drift, int drift_axis,
                      double u_thi, double u_the, cudaStream_t s);
void mix3_energy(const Dev3D& d, cudaStream_t s);
void mix3_moments(const Dev3D& d, const Mix3Const& k, double* mom, cudaStream_t s);

void curre_fold3d(const Dev3D& d, cudaStream_t s);
void bc_mom3d(const Dev3D& d, double* mom, cudaStream_t s);
void injection3d(const Dev3D& d, const Parts3D& P, double u0, double xend, cudaStream_t s);
void dfield_ghost3d(const Dev3D& d, cudaStream_t s);
void uf_add3d(const Dev3D& d, cudaStream_t s);
void particle_x3d(const Dev3D& d, const Parts3D& P, cudaStream_t s);
void migrate_scan3d(const Dev3D& d, const Parts3D& P, cudaStream_t s);
void migrate_plan3d(const Dev3D& d, cudaStream_t s);
void sort_rank3d(const Dev3D& d, const Parts3D& P, const int* slist, cudaStream_t s);
void gather3d(const Dev3D& d, const Parts3D& src, const Parts3D& dst, const int* map, const int* counts,
              cudaStream_t s);
void aos_to_soa3d(const Dev3D& d, const double* aos, int ndim, int np_host, int row0, int nrows, const Parts3D& P,
                  cudaStream_t s);
void soa_to_aos3d(const Dev3D& d, double* aos, int ndim, int np_host, int row0, int nrows, const Parts3D& P,
                  cudaStream_t s);
void load_weibel3d_ppc(const Dev3D& d, int ppc, unsigned long long seed, double drift, int drift_axis,
                       double u_thi, double u_the, cudaStream_t s);

}  // namespace wpic
