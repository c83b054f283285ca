/*
 * wumingpic_gb300.h -- C ABI of the GB300 (sm_103a) implementation of WumingPIC's
 * particle-in-cell time step.
 *
 * The library replaces, for one GPU holding the whole domain, the module
 * procedures that WumingPIC's Fortran drivers ({2d,3d}/proj/STAR/app.f90) call every
 * step.  Each entry point below names the reference procedure it stands in for.
 * All arrays passed across this boundary use the reference's own layout
 * (Fortran column-major, the lower bounds of the Fortran declarations):
 *
 *   2D  up, gp     real(8) (ndim, np, nys:nye, nsp)              ndim = 6: x, y, ux, uy, uz, id
 *       uf         real(8) (6, nxgs-2:nxge+2, nys-2:nye+2)        Bx, By, Bz, Ex, Ey, Ez
 *       uj         real(8) (3, nxgs-2:nxge+2, nys-2:nye+2)
 *       df         real(8) (6, nxgs-2:nxge+2, nys-2:nye+2)        CG warm start / field increment
 *       cumcnt     integer (nxgs:nxge+1, nys:nye, nsp)
 *       np2        integer (nys:nye, nsp)
 *
 * The particle id slot holds the 64-bit integer id bit-cast into a real(8)
 * (2d/proj/weibel/app.f90:468) and is carried bit for bit.
 *
 * State lives on the device between calls (the caller's arrays are read by
 * wpic_put_* and written by wpic_get_*).  Every function returns a status code
 * instead of stopping the program as the reference does; none of them aborts.
 * One host thread per context; all work is ordered on the context's stream.
 */
#ifndef WUMINGPIC_GB300_H
#define WUMINGPIC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define WPIC_OK 0
#define WPIC_CG_NOT_CONVERGED 1 /* reference: 'stop at cgm after ite_max' (2d/common/field.f90:427-430) */
#define WPIC_CAPACITY 2         /* reference: 'memory over (np2 > np)' (2d/common/boundary_periodic.f90:231-234) */
#define WPIC_OUT_OF_RANGE 3     /* a particle outside the domain where the reference indexes out of bounds */
#define WPIC_MOVED_TOO_FAR 4    /* a particle crossed more than one cell in one step (c*dt >= dx) */
#define WPIC_NONFINITE 5
#define WPIC_BAD_ARGUMENT 6
#define WPIC_CUDA_ERROR 7
#define WPIC_NOT_INITIALISED 8
#define WPIC_STAGING_TIMEOUT 9  /* a bulk copy into shared memory did not complete within the kernel's
                                   bounded wait; the copy may have been left in flight, so finalise
                                   the context instead of stepping it again */

/* boundary kinds: replace the procedure arguments of field__fdtd_i
 * (2d/common/field.f90:66-89) and the driver's choice of boundary module */
#define WPIC_BC_PERIODIC 0     /* boundary_periodic (2d/common/boundary_periodic.f90) */
#define WPIC_BC_RECONNECTION 1 /* boundary_reconnection: conducting walls in x
                                  (2d/proj/reconnection/boundary_reconnection.f90) */
#define WPIC_BC_SHOCK 2        /* boundary_shock: reflecting wall at nxs, injection boundary at
                                  nxe of the active window (2d/proj/shock/boundary_shock.f90);
                                  FP64 paths */

/* arithmetic of the particle and field kernels */
#define WPIC_FP64 0       /* FP64, fused multiply-add allowed */
#define WPIC_FP64_EXACT 1 /* FP64 in the reference's operation order (bit-exact parity mode) */
#define WPIC_MIXED 2      /* positions as integer cell + FP32 offset, FP32 push / gather / deposition
                             weights, FP32 tile currents flushed into FP64 J, FP64 field solve.
                             Requires nx and ny to be multiples of 16; particles live in 16 x 16-cell
                             tile bins whose capacity is np * 256 / nx slots per species.  The drivers'
                             staged calls map onto the fused step (see wpic_particle_solv), and the
                             state exchange keeps only the sorted state (see wpic_put_particles). */

/* the push of the fused step: particle__solv (Buneman-Boris) or particle__solv_vay */
#define WPIC_PUSH_BORIS 0
#define WPIC_PUSH_VAY 1   /* every path; the mixed paths run it inside their fused step */

typedef struct wpic_ctx wpic_ctx;

/* The scalar arguments of particle__init (2d/common/particle.f90:18-45),
 * field__init (2d/common/field.f90:22-63), sort__init (2d/common/sort.f90:16-33)
 * and bc__init (2d/common/boundary_periodic.f90:26-58), merged.  With one GPU
 * holding the whole domain nys = nygs and nye = nyge. */
typedef struct wpic_params {
  int ndim;                 /* 6 in 2D */
  int np;                   /* per-row capacity of the caller's particle arrays */
  int nsp;                  /* number of species, 1 or 2 */
  int nxgs, nxge, nygs, nyge, nys, nye;
  double delx, delt, c, gfac;
  double q[2], r[2];        /* charge and mass of each species */
  int bc_kind;              /* WPIC_BC_* */
  int precision;            /* WPIC_FP64, WPIC_FP64_EXACT or WPIC_MIXED */
  int device_cap;           /* device particle slots per row per species; 0 = np */
} wpic_params;

/* particle__init + field__init + sort__init + bc__init for a 2D run.
 * cuda_stream: a cudaStream_t to order all work on, or NULL for a private stream. */
int wpic_init_2d(wpic_ctx** ctx, const wpic_params* p, void* cuda_stream);
int wpic_finalize(wpic_ctx* ctx);

/* State exchange in the reference layout.  which = 0: the sorted state 'up'
 * with its cumcnt; which = 1: the scratch/new state 'gp' (cumcnt ignored).
 * np2 is shared by both.  put validates np2 <= device capacity and the cumcnt
 * prefix sums.  A mixed context keeps only the sorted state: put with which = 1 takes the
 * unsorted rows of the restart path (io__input, before sort__bucket), sorts each row by x cell
 * on the host and stores it as the sorted state. */
int wpic_put_particles(wpic_ctx* ctx, int which, const double* up, const int* np2, const int* cumcnt);
int wpic_get_particles(wpic_ctx* ctx, int which, double* up, int* np2, int* cumcnt);
int wpic_put_fields(wpic_ctx* ctx, const double* uf);
int wpic_get_fields(wpic_ctx* ctx, double* uf);
/* The SAVEd field__fdtd_i arrays (2d/common/field.f90:98): df is the CG warm
 * start carried from step to step; uj is the current after the boundary fold. */
int wpic_put_df(wpic_ctx* ctx, const double* df);
int wpic_get_df(wpic_ctx* ctx, double* df);
int wpic_get_uj(wpic_ctx* ctx, double* uj);

/* The drivers' staged calls.  On a WPIC_MIXED context they map onto the fused mixed step:
 * particle__solv (or _vay) requests the push, field__fdtd_i runs the whole step (push, deposit,
 * x boundary, cell-leavers into their columns, field solve), and bc__particle_x,
 * bc__particle_y and sort__bucket find their work done; the Weibel order (push, field,
 * particle_x) and the reconnection order (push, particle_x, field) are both accepted, and a
 * shock context takes boundary_shock__injection's u0 between the push and the field solve.
 * Out of order (a field solve without its push, a second push, particle_y or sort__bucket
 * between push and field solve) they return WPIC_BAD_ARGUMENT.
 * particle__solv(gp, up, uf, cumcnt, nxs, nxe)      2d/common/particle.f90:48-179 */
int wpic_particle_solv(wpic_ctx* ctx);
/* particle__solv_vay(gp,up,uf,cumcnt,nxs,nxe)  2d/common/particle.f90:182 */
int wpic_particle_solv_vay(wpic_ctx* ctx);
/* which push the fused step (wpic_step) uses: WPIC_PUSH_BORIS (default) or WPIC_PUSH_VAY */
int wpic_set_pusher(wpic_ctx* ctx, int pusher);
/* the active x window nxs..nxe that the drivers pass to every module call; the shock
 * driver widens it as its box expands (2d/proj/shock/app.f90:276-277, 615-625).  Default:
 * the whole domain; non-periodic contexts only (on the mixed path, shock only).  Cells
 * outside the window hold no particles and keep their fields. */
int wpic_set_window(wpic_ctx* ctx, int nxs, int nxe);
/* the upstream four-velocity u0 of boundary_shock__injection used by the fused step */
int wpic_set_injection(wpic_ctx* ctx, double u0);
/* boundary_shock__injection(gp,np2,nxs,nxe,u0)   2d/proj/shock/boundary_shock.f90:255 */
int wpic_bc_injection(wpic_ctx* ctx, double u0);

/* Moments (the driver's diagnostic block, 2d/proj/weibel/app.f90:121-123).  The device keeps
 * mom(7, nxgs-1:nxge+1, nys-1:nye+1, nsp) in the reference's layout: number density, the three
 * velocity components and the diagonal of u v at the half-integer nodes, per species.  On a
 * mixed context mom_calc__nvt (from_gp = 1) computes the folded moments with the FP32
 * half-step push, and mom_calc__accl and bc__mom have nothing left to do.
 * mom_calc__accl(gp,up,uf,cumcnt,nxs,nxe)   2d/common/mom_calc.f90:48   (FP64 paths): writes gp */
int wpic_mom_calc_accl(wpic_ctx* ctx);
/* mom_calc__nvt(mom,gp,np2)   2d/common/mom_calc.f90:164; from_gp = 1 reads gp (after
 * wpic_mom_calc_accl), 0 reads up.  The particles must be bucket-sorted (cumcnt). */
int wpic_mom_calc_nvt(wpic_ctx* ctx, int from_gp);
/* bc__mom(mom): boundary_periodic__mom 2d/common/boundary_periodic.f90:571,
 * boundary_reconnection__mom 2d/proj/reconnection/boundary_reconnection.f90:582 */
int wpic_bc_mom(wpic_ctx* ctx);
/* the device moments to a host array of 7*(nx+2)*(ny+2)*nsp doubles */
int wpic_get_mom(wpic_ctx* ctx, double* mom);
/* accl + nvt + bc__mom in one call (all paths; the mixed path computes the half-step push in
 * FP32 and leaves the particle state untouched); mom may be NULL to keep the result on the device */
int wpic_moments(wpic_ctx* ctx, double* mom);
/* field__fdtd_i(uf, up, gp, cumcnt, nxs, nxe, bc__dfield, bc__curre, bc__phi)
 *                                                   2d/common/field.f90:66-186 */
int wpic_field_fdtd_i(wpic_ctx* ctx);
/* ele_cur + bc__curre only (the current that field__fdtd_i deposits), for checks
 *                                                   2d/common/field.f90:189-316 */
int wpic_ele_cur(wpic_ctx* ctx);
/* bc__particle_x(gp, np2)                           2d/common/boundary_periodic.f90:61-96
 *                                                   2d/proj/reconnection/boundary_reconnection.f90:61-99 */
int wpic_bc_particle_x(wpic_ctx* ctx);
/* bc__particle_y(gp, np2)                           2d/common/boundary_periodic.f90:99-248 */
int wpic_bc_particle_y(wpic_ctx* ctx);
/* sort__bucket(up, gp, cumcnt, np2, nxs, nxe)       2d/common/sort.f90:36-82 */
int wpic_sort_bucket(wpic_ctx* ctx);
/* nsteps iterations of the driver loop body (2d/proj/weibel/app.f90:102-107;
 * reconnection order 2d/proj/reconnection/app.f90:101-106), fused. */
int wpic_step(wpic_ctx* ctx, int nsteps);

/* energy_history sums (2d/proj/weibel/app.f90:502-534):
 * out[0..nsp-1] = sum r (gamma-1) per species, out[nsp] = sum E^2 / 8pi, out[nsp+1] = sum B^2 / 8pi */
int wpic_energy(wpic_ctx* ctx, double* out);

/* CG control: fixed3[l] >= 0 runs exactly that many iterations for component l
 * (parity mode), < 0 or fixed3 == NULL uses the reference stopping rule;
 * ite_max as in cgm (2d/common/field.f90:337).  cg_iters returns the last counts. */
int wpic_cg_control(wpic_ctx* ctx, const int* fixed3, int ite_max);
int wpic_cg_iters(wpic_ctx* ctx, int* out3);
/* the CG stopping tolerance relative to ||b|| (the reference's 1e-6, field.f90:364) and the
 * iteration limit (100, field.f90:427); a tight tolerance for gradient checks */
int wpic_cg_tolerance(wpic_ctx* ctx, double rtol, int ite_max);

/* Discrete adjoint of nsteps fused steps from the current state (FP64 paths, periodic, the
 * Boris push): given lam_uf_final, the gradient of a scalar with respect to the fields after
 * the last step (reference layout uf(6, nxgs-2:nxge+2, nys-2:nye+2)), returns its gradient with
 * respect to the particles (lam_up0, layout of up with the ids in the id column) and the fields
 * (lam_uf0) at the start.  States are kept every `every` steps and recomputed in between.
 * The context is left in its state after the nsteps steps. */
int wpic_adjoint(wpic_ctx* ctx, int nsteps, int every, const double* lam_uf_final, double* lam_up0,
                 double* lam_uf0);
/* wpic_adjoint in two halves.  record: nsteps steps from the current state, keeping the state
 * at every segment start and at the end.  reverse: the gradients for the recorded run (may be
 * called again with another lam_uf_final); leaves the recorded final state in the context. */
int wpic_adjoint_record(wpic_ctx* ctx, int nsteps, int every);
/* arithmetic of the reverse push and deposit sweeps: WPIC_FP64 (default) or WPIC_MIXED (FP32
   per particle along the recorded FP64 trajectory; fields, adjoint CG and sums stay FP64) */
int wpic_adjoint_precision(wpic_ctx* ctx, int precision);
/* keep (1, default) or not (0) the field state of every recorded step, 12 field planes of
   doubles per step, when that fits in half of the free device memory: the reverse sweep's
   recompute of a segment then pushes and sorts only, with the recorded fields replayed
   (the same particle states as a full recompute, bit for bit).  Read by the next record;
   0 also frees the store, after which a recorded run is recomputed in full. */
int wpic_adjoint_keep_fields(wpic_ctx* ctx, int keep);
int wpic_adjoint_reverse(wpic_ctx* ctx, const double* lam_uf_final, double* lam_up0, double* lam_uf0);
/* dot-product checks <L x, y> = <x, L^T y> of the adjoint's transposed field operators on
 * random vectors (current fold, ghost copies, E update, RHS, cell-centre averaging): five
 * relative differences.  Overwrites the context's fields. */
int wpic_adjoint_selfcheck(wpic_ctx* ctx, double* out5);
/* the push's field adjoint against a central difference of the push along a random field
 * direction (step hstep), both projected on random particle adjoints: out2 = {difference,
 * adjoint} */
int wpic_adjoint_pushcheck(wpic_ctx* ctx, double hstep, double* out2);
/* the deposit's adjoint against a central difference along random particle directions */
int wpic_adjoint_depositcheck(wpic_ctx* ctx, double hstep, double* out2);
/* the fields -> push -> deposit chain's adjoint against a central difference along random fields */
int wpic_adjoint_chaincheck(wpic_ctx* ctx, double hstep, double* out2);

/* Device-side seeded loader of a 2D Weibel plasma (no reference counterpart:
 * the reference loads on the host from an unseeded RNG, 2d/proj/weibel/app.f90:380-437). */
int wpic_load_weibel_2d(wpic_ctx* ctx, int ppc, uint64_t seed, double drift, int drift_axis, double u_thi,
                        double u_the, const double* b0);

/* Stage timing with CUDA events on the context stream: enable != 0 starts
 * accumulating; times returns ms per stage and launch counts (see wpic_stage_name). */
int wpic_timing_enable(wpic_ctx* ctx, int enable);
int wpic_timing_get(wpic_ctx* ctx, double* ms, long long* launches, int n);
const char* wpic_stage_name(int stage);
int wpic_num_stages(void);

/* FMA throughput of the device in GFLOP/s (fp64 != 0: FP64, else FP32), measured by a
 * register-only kernel; the compute roof the FP64 kernels are reported against. */
int wpic_measure_fma_peak(int fp64, double* gflops);

/* Page-lock and map (and release) a caller's host array, e.g. the reference-layout up/uf
 * arrays, so that wpic_put_* / wpic_get_* move it at full host-link bandwidth; on a mixed 2D
 * context the conversion kernels then read and write the registered particle array in place
 * (when it is 16-byte aligned, as malloc and Fortran allocations are; otherwise staged copies). */
int wpic_host_register(void* ptr, size_t bytes);
int wpic_host_unregister(void* ptr);

/* The energy_history sums of wpic_energy, computed from the caller's own device
 * arrays without allocating anything.  No counterpart in the reference.
 *
 * For callers that cannot allocate device memory where they need the diagnostic:
 * arrays held on the device by another runtime's allocator (OpenACC or CUDA Fortran
 * data regions, a framework's pool), a time-step loop where cudaMalloc would
 * synchronise the device, or a run sized to fill HBM.  up (ndim, np, ny, nsp),
 * np2 (ny, nsp) and uf (6, nx+4, ny+4) are device pointers in the reference layout;
 * r holds the nsp masses in host memory; out is a device pointer to nsp+2 doubles,
 * laid out as in wpic_energy.  Work is queued on stream (NULL: the default stream)
 * and out is valid once the stream reaches it.
 *
 * Scratch: a fixed __device__ array of 3 * WPIC_NOALLOC_MAX_ROWS doubles (192 KiB)
 * that every GPU loading the library holds until the process exits.  Grids with
 * ny * nsp > WPIC_NOALLOC_MAX_ROWS are refused with WPIC_BAD_ARGUMENT.  All calls
 * share the array, so calls that overlap on the GPU race.  The first call on each
 * device looks up the array's device address; make that first call before any
 * stream capture.  The address is kept for the life of the process: after a
 * cudaDeviceReset the library's device code is loaded again in a new context, where
 * the array may lie elsewhere, so do not call this entry point after resetting a
 * device. */
#define WPIC_NOALLOC_MAX_ROWS 8192
int wpic_energy_noalloc(const double* up, const int* np2, const double* uf, int ndim, int np, int nx, int ny,
                        int nsp, const double* r, double c, double* out, void* stream);

int wpic_synchronize(wpic_ctx* ctx);
long long wpic_num_particles(wpic_ctx* ctx);
const char* wpic_status_string(int status);

/* ------------------------------------------------------------------------- */
/* 3D (periodic in x, y and z), FP64 path.  The arrays follow the 3D drivers:  */
/*   up/gp(7, np, nys:nye, nzs:nze, nsp): x, y, z, ux, uy, uz, id (bit-cast)  */
/*   uf(6, nxgs-2:nxge+2, nys-2:nye+2, nzs-2:nze+2), cumcnt(nxgs:nxge+1,       */
/*   nys:nye, nzs:nze, nsp), np2(nys:nye, nzs:nze, nsp).                        */
/* nx, ny, nz >= 4; one device holds the whole domain (nys = nygs, ...).       */
/* ------------------------------------------------------------------------- */
typedef struct wpic_ctx3d wpic_ctx3d;

typedef struct wpic_params3d {
  int ndim;                 /* 7 in 3D */
  int np;                   /* per-row capacity of the caller's particle arrays */
  int nsp;                  /* 1 or 2 */
  int nxgs, nxge, nygs, nyge, nzgs, nzge, nys, nye, nzs, nze;
  double delx, delt, c, gfac;
  double q[2], r[2];
  int precision;            /* WPIC_FP64, WPIC_FP64_EXACT or WPIC_MIXED */
  int device_cap;           /* device particle slots per row per species; 0 = np */
  int bc_kind;              /* WPIC_BC_PERIODIC (3d/common/boundary_periodic.f90), WPIC_BC_RECONNECTION:
                               conducting walls in x, 3d/proj/reconnection/boundary_reconnection.f90,
                               or WPIC_BC_SHOCK: 3d/proj/shock/boundary_shock.f90 (FP64 paths) */
} wpic_params3d;

/* particle__init + field__init + sort__init + bc__init of a 3D run
   (3d/common/particle.f90:18, field.f90:22, sort.f90:18, boundary_periodic.f90:25) */
int wpic3d_init(wpic_ctx3d** ctx, const wpic_params3d* p, void* cuda_stream);
int wpic3d_finalize(wpic_ctx3d* ctx);
/* which = 0: up (with cumcnt), 1: gp (on a mixed context: the unsorted rows of the restart
 * path, sorted by x cell on the host into the sorted state) */
int wpic3d_put_particles(wpic_ctx3d* ctx, int which, const double* up, const int* np2, const int* cumcnt);
int wpic3d_get_particles(wpic_ctx3d* ctx, int which, double* up, int* np2, int* cumcnt);
int wpic3d_put_fields(wpic_ctx3d* ctx, const double* uf);
int wpic3d_get_fields(wpic_ctx3d* ctx, double* uf);
/* the CG warm start of field__fdtd_i (SAVEd df), for a restart that continues bit for bit */
int wpic3d_put_df(wpic_ctx3d* ctx, const double* df);
int wpic3d_get_df(wpic_ctx3d* ctx, double* df);   /* the SAVEd dB/dE of field__fdtd_i */
int wpic3d_get_uj(wpic_ctx3d* ctx, double* uj);   /* the current of the last field__fdtd_i */
/* The staged calls map onto the fused mixed step on a WPIC_MIXED context as in 2D:
 * particle__solv (or _vay) requests the push, field__fdtd_i runs the step, bc__particle_x,
 * bc__particle_yz and sort__bucket find their work done, boundary_shock__injection between
 * the push and the field solve sets u0, mom_calc__nvt (from gp) computes the folded moments.
 * particle__solv(gp, up, uf, cumcnt, nxs, nxe)       3d/common/particle.f90:52 */
int wpic3d_particle_solv(wpic_ctx3d* ctx);
/* particle__solv_vay(gp, up, uf, cumcnt, nxs, nxe)   3d/common/particle.f90:236 */
int wpic3d_particle_solv_vay(wpic_ctx3d* ctx);
int wpic3d_set_pusher(wpic_ctx3d* ctx, int pusher);
/* mom_calc__accl  3d/common/mom_calc.f90:49; mom_calc__nvt  3d/common/mom_calc.f90:219;
 * bc__mom = boundary_periodic__mom  3d/common/boundary_periodic.f90:1102;
 * mom(7, nxgs-1:nxge+1, nys-1:nye+1, nzs-1:nze+1, nsp) */
int wpic3d_mom_calc_accl(wpic_ctx3d* ctx);
int wpic3d_mom_calc_nvt(wpic_ctx3d* ctx, int from_gp);
int wpic3d_bc_mom(wpic_ctx3d* ctx);
int wpic3d_get_mom(wpic_ctx3d* ctx, double* mom);
int wpic3d_moments(wpic_ctx3d* ctx, double* mom);
/* field__fdtd_i(uf, up, gp, cumcnt, nxs, nxe, ...)   3d/common/field.f90:70 */
int wpic3d_field_fdtd_i(wpic_ctx3d* ctx);
/* ele_cur + bc__curre, the deposit half of field__fdtd_i (3d/common/field.f90:129-130) */
int wpic3d_ele_cur(wpic_ctx3d* ctx);
/* bc__particle_x(gp, np2)                            3d/common/boundary_periodic.f90:68 */
int wpic3d_bc_particle_x(wpic_ctx3d* ctx);
/* bc__particle_yz(gp, np2)                           3d/common/boundary_periodic.f90:104 */
int wpic3d_bc_particle_yz(wpic_ctx3d* ctx);
/* the shock run (bc_kind WPIC_BC_SHOCK, FP64 paths; 3d/proj/shock): the active x window nxs..nxe
 * every module call receives (3d/proj/shock/app.f90:112-117, widened by relocate at :654), the
 * injection boundary's upstream four-velocity u0 for wpic3d_step, and
 * boundary_shock__injection(gp,np2,nxs,nxe,u0) (3d/proj/shock/boundary_shock.f90:424) on gp */
int wpic3d_set_window(wpic_ctx3d* ctx, int nxs, int nxe);
int wpic3d_set_injection(wpic_ctx3d* ctx, double u0);
int wpic3d_bc_injection(wpic_ctx3d* ctx, double u0);
/* sort__bucket(up, gp, cumcnt, np2, nxs, nxe)        3d/common/sort.f90:40 */
int wpic3d_sort_bucket(wpic_ctx3d* ctx);
/* the driver loop body (3d/proj/weibel/app.f90:103-108), nsteps times */
int wpic3d_step(wpic_ctx3d* ctx, int nsteps);
/* energy_history sums (3d/proj/weibel/app.f90:531-566): kinetic per species, E, B */
int wpic3d_energy(wpic_ctx3d* ctx, double* out);
int wpic3d_cg_control(wpic_ctx3d* ctx, const int* fixed3, int ite_max);
int wpic3d_cg_iters(wpic_ctx3d* ctx, int* out3);
/* seeded synthetic Weibel plasma (no counterpart in the reference: its loader is unseeded) */
int wpic3d_load_weibel(wpic_ctx3d* ctx, int ppc, uint64_t seed, double drift, int drift_axis, double u_thi,
                       double u_the);
long long wpic3d_num_particles(wpic_ctx3d* ctx);
int wpic3d_synchronize(wpic_ctx3d* ctx);

#ifdef __cplusplus
}
#endif

#endif /* WUMINGPIC_GB300_H */
