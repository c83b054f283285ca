// C ABI of the 3D FP64 path (declared in include/wumingpic_gb300.h): context
// creation, device memory, reference-layout state exchange, and the host-side
// sequencing of one 3D time step (3d/proj/weibel/app.f90:103-108).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "wumingpic_gb300.h"
#include "wpic_internal.h"

using namespace wpic;

struct wpic_ctx3d {
  wpic_params3d prm;
  Dev3D d;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  CGState* h_cg = nullptr;
  int* h_err = nullptr;
  int cg_fixed[3] = {-1, -1, -1};
  int cg_pred = 4;  // iterations enqueued before the first host check: the last solve's count
  int cg_iters[3] = {0, 0, 0};
  std::vector<void*> allocs;
  double* staging = nullptr;
  size_t staging_bytes = 0;
  int pusher = WPIC_PUSH_BORIS;  // the push of the fused step
  double u0 = 0.0;               // shock runs: the upstream four-velocity of the injection boundary
  double* mom = nullptr;         // mom(7, nxgs-1:nxge+1, nys-1:nye+1, nzs-1:nze+1, nsp), on first use
  bool mixed = false;            // FP32 push/deposit on split positions (the fused step)
  // the drivers' staged calls on a mixed context: particle__solv asks for the push
  // (mix_pending, with its pusher) and field__fdtd_i runs the fused mixed step
  bool mix_pending = false;
  int mix_pending_pusher = WPIC_PUSH_BORIS;
  Mix3Const mk{};
  alignas(128) unsigned char tmap[128];  // CUtensorMap of uf (mixed path TMA tile loads)
  // mixed path: the particle layers (reallocated when bins grow) and the host copy of the layout
  float* mixP = nullptr;
  int* mixK = nullptr;           // the arrival keys of the layout (one per slot)
  std::vector<int> h_dep;
  int* h_grow = nullptr;         // pinned mirror of the grow flag
  double mix_vmax = 0.0;         // largest contribution of one particle to one node of the deposit
};

namespace {

constexpr int CG3_CHECK_EVERY = 4;
constexpr int CG_THREADS_HOST = 256;  // threads of the CG reduction blocks

int cuda_status3(cudaError_t e) {
  if (e == cudaSuccess) return WPIC_OK;
  fprintf(stderr, "wumingpic_gb300: CUDA error %s\n", cudaGetErrorString(e));
  return WPIC_CUDA_ERROR;
}

#define CK3(call)                                   \
  do {                                              \
    cudaError_t e_ = (call);                        \
    if (e_ != cudaSuccess) return cuda_status3(e_); \
  } while (0)

template <typename T>
int dalloc3(wpic_ctx3d* c, T** p, size_t n) {
  void* v = nullptr;
  cudaError_t e = cudaMalloc(&v, n * sizeof(T) + 16);
  if (e != cudaSuccess) return cuda_status3(e);
  c->allocs.push_back(v);
  e = cudaMemsetAsync(v, 0, n * sizeof(T) + 16, c->stream);
  if (e != cudaSuccess) return cuda_status3(e);
  *p = (T*)v;
  return WPIC_OK;
}

int alloc_parts3(wpic_ctx3d* c, Parts3D* P, size_t n) {
  int st;
  if ((st = dalloc3(c, &P->x, n)) || (st = dalloc3(c, &P->y, n)) || (st = dalloc3(c, &P->z, n)) ||
      (st = dalloc3(c, &P->ux, n)) || (st = dalloc3(c, &P->uy, n)) || (st = dalloc3(c, &P->uz, n)) ||
      (st = dalloc3(c, &P->id, n)))
    return st;
  return WPIC_OK;
}

int finish3(wpic_ctx3d* c) {
  cudaError_t e = cudaMemcpyAsync(c->h_err, c->d.err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status3(e);
  const int bits = *c->h_err;
  if (bits) cudaMemsetAsync(c->d.err, 0, sizeof(int), c->stream);
  if (bits & EB_STAGING_TIMEOUT) return WPIC_STAGING_TIMEOUT;
  if (bits & EB_MOVED_TOO_FAR) return WPIC_MOVED_TOO_FAR;
  if (bits & EB_OUT_OF_RANGE) return WPIC_OUT_OF_RANGE;
  if (bits & EB_CAPACITY) return WPIC_CAPACITY;
  if (bits & EB_CG) return WPIC_CG_NOT_CONVERGED;
  return WPIC_OK;
}

bool exact3(const wpic_ctx3d* c) { return c->prm.precision == WPIC_FP64_EXACT; }

#define FP3(fn, ...)                            \
  do {                                          \
    if (exact3(c)) exact::fn(__VA_ARGS__);      \
    else fast::fn(__VA_ARGS__);                 \
  } while (0)

int ensure_staging3(wpic_ctx3d* c, size_t bytes) {
  if (c->staging_bytes >= bytes) return WPIC_OK;
  if (c->staging) {
    cudaStreamSynchronize(c->stream);
    cudaFree(c->staging);
    c->staging = nullptr;
    c->staging_bytes = 0;
  }
  CK3(cudaMalloc(&c->staging, bytes));
  c->staging_bytes = bytes;
  return WPIC_OK;
}

int do_cg3(wpic_ctx3d* c) {
  for (int l = 0; l < 3; ++l) c->h_cg[l].fixed = c->cg_fixed[l];
  for (int l = 0; l < 3; ++l)
    CK3(cudaMemcpyAsync(&c->d.cg[l].fixed, &c->h_cg[l].fixed, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  FP3(cg_init3d, c->d, c->stream);
  // the iterations run on device flags; the host enqueues the last solve's count first, then
  // CG3_CHECK_EVERY at a time until every component has stopped
  int chunk = c->cg_pred;
  for (int guard = 0; guard < 100000; ++guard) {
    for (int k = 0; k < chunk; ++k) {
      FP3(cg_iter_ap3d, c->d, c->stream);
      FP3(cg_iter_update3d, c->d, c->stream);
      FP3(cg_iter_p3d, c->d, c->stream);
    }
    CK3(cudaMemcpyAsync(c->h_cg, c->d.cg, 3 * sizeof(CGState), cudaMemcpyDeviceToHost, c->stream));
    CK3(cudaStreamSynchronize(c->stream));
    if (!c->h_cg[0].active && !c->h_cg[1].active && !c->h_cg[2].active) break;
    chunk = CG3_CHECK_EVERY;
  }
  int most = 1;
  for (int l = 0; l < 3; ++l) {
    c->cg_iters[l] = c->h_cg[l].ite;
    most = std::max(most, c->h_cg[l].ite);
  }
  c->cg_pred = std::min(most, 100);
  FP3(cg_store3d, c->d, c->stream);
  return WPIC_OK;
}

// field__fdtd_i (3d/common/field.f90:70-208)
int do_field3(wpic_ctx3d* c) {
  FP3(deposit3d, c->d, c->stream);  // ele_cur
  curre_fold3d(c->d, c->stream);
  FP3(gkl3d, c->d, c->stream);
  int st = do_cg3(c);
  if (st) return st;
  dfield_ghost3d(c->d, c->stream);
  FP3(efield3d, c->d, c->stream);
  dfield_ghost3d(c->d, c->stream);
  uf_add3d(c->d, c->stream);
  return WPIC_OK;
}

// bc__particle_yz + sort__bucket fused: B (pushed, x-wrapped) -> A (migrated and sorted)
void do_migrate_sort3(wpic_ctx3d* c) {
  migrate_scan3d(c->d, c->d.B, c->stream);
  migrate_plan3d(c->d, c->stream);
  sort_rank3d(c->d, c->d.B, c->d.slist, c->stream);
  gather3d(c->d, c->d.B, c->d.A, c->d.map, c->d.np2new, c->stream);
  cudaMemcpyAsync(c->d.np2, c->d.np2new, sizeof(int) * c->d.nrow, cudaMemcpyDeviceToDevice, c->stream);
}

// Fixed-point scales of the mixed deposit for columns of at most maxdep slots.  One particle adds
// at most vmax = max |q| dx/dt to a node; a thread flushes the sum of up to 32 particles at once
// (|v s1| <= 2^21 keeps the magic-number rounding exact), at most 125 * nsp * maxdep particles
// reach a node in one tile pass (|sum hi| < 2^30), and each of them adds at most 2^14 to the low
// plane.  The current is rebuilt every step, so the scales may change with the layout.
int mix3_set_scales(wpic_ctx3d* c, int maxdep) {
  Mix3D& m = c->d.m;
  const double vmax = c->mix_vmax;
  const double reach = 125.0 * c->prm.nsp * maxdep;
  double s1 = std::ldexp(1.0, 21) / (32.0 * vmax);
  const double lim = std::ldexp(1.0, 30) / (reach * vmax);
  if (lim < s1) s1 = lim;
  s1 = std::ldexp(1.0, (int)std::floor(std::log2(s1)));
  if (!(s1 > 0.0) || s1 > std::ldexp(1.0, 100) || (reach + 27.0) * 16384.0 >= std::ldexp(1.0, 31))
    return WPIC_CAPACITY;
  m.fx_s1 = (float)s1;
  m.fx_is1f = (float)(1.0 / s1);
  m.fx_s2 = (float)(s1 * 32768.0);
  m.fx_is2 = 1.0 / (s1 * 32768.0);
  return WPIC_OK;
}

// Lays the mixed-path bins out with the given depths.  keep = true copies the columns of the
// current layout (counts unchanged); otherwise the new layout starts empty.
int mix3_set_layout(wpic_ctx3d* c, const std::vector<int>& dep, bool keep) {
  Mix3D& m = c->d.m;
  std::vector<long long> off(m.nbin);
  long long layers = 0;
  int maxdep = 1;
  for (int b = 0; b < m.nbin; ++b) {
    if (dep[b] < 1 || dep[b] > MIX_MAX_DEPTH) return WPIC_CAPACITY;
    off[b] = layers;
    layers += dep[b];
    maxdep = std::max(maxdep, dep[b]);
  }
  if (int st = mix3_set_scales(c, maxdep)) return st;
  if (!keep && c->mixP) {
    CK3(cudaStreamSynchronize(c->stream));
    cudaFree(c->mixP);
    c->mixP = nullptr;
  }
  // the keys only pass from a push to the arrival kernel: the old ones are not kept
  CK3(cudaStreamSynchronize(c->stream));
  if (c->mixK) cudaFree(c->mixK);
  c->mixK = nullptr;
  CK3(cudaMalloc(&c->mixK, (size_t)layers * M3_TC * sizeof(int)));
  m.K = c->mixK;
  float* np_ = nullptr;
  CK3(cudaMalloc(&np_, (size_t)layers * M3_PL * sizeof(float)));
  long long* old_off = nullptr;
  const float* old_P = c->mixP;
  if (keep && old_P) {
    CK3(cudaMalloc(&old_off, sizeof(long long) * m.nbin));
    CK3(cudaMemcpyAsync(old_off, m.boff, sizeof(long long) * m.nbin, cudaMemcpyDeviceToDevice, c->stream));
  }
  CK3(cudaMemcpyAsync(m.boff, off.data(), sizeof(long long) * m.nbin, cudaMemcpyHostToDevice, c->stream));
  CK3(cudaMemcpyAsync(m.bdep, dep.data(), sizeof(int) * m.nbin, cudaMemcpyHostToDevice, c->stream));
  m.P = np_;
  if (keep && old_P) mix3_relayout(c->d, old_P, old_off, c->stream);
  CK3(cudaStreamSynchronize(c->stream));  // host vectors and the old buffers are released below
  if (old_off) cudaFree(old_off);
  if (keep && old_P) cudaFree(c->mixP);
  c->mixP = np_;
  c->h_dep = dep;
  return WPIC_OK;
}

// grows the bins whose columns came within 1/8 of full in the last step to 1.5 x their need
int mix3_grow(wpic_ctx3d* c) {
  Mix3D& m = c->d.m;
  std::vector<int> need(m.nbin);
  CK3(cudaMemcpyAsync(need.data(), m.bneed, sizeof(int) * m.nbin, cudaMemcpyDeviceToHost, c->stream));
  CK3(cudaMemsetAsync(m.grow, 0, sizeof(int), c->stream));
  CK3(cudaStreamSynchronize(c->stream));
  *c->h_grow = 0;
  std::vector<int> dep = c->h_dep;
  bool any = false;
  for (int b = 0; b < m.nbin; ++b)
    if (8LL * need[b] > 7LL * dep[b]) {
      const long long nd = ((long long)std::ceil(1.5 * need[b] + 8.0) + 7) & ~7LL;
      dep[b] = (int)(nd > MIX_MAX_DEPTH ? MIX_MAX_DEPTH : nd);
      any = true;
    }
  return any ? mix3_set_layout(c, dep, true) : WPIC_OK;
}

double shock_xend3(const wpic_ctx3d* c, double u0);

// the mixed step: fused FP32 push + deposit + compaction, the arrivals, then the FP64 field solve
int mixed_step3(wpic_ctx3d* c) {
  Dev3D& d = c->d;
  if (d.ph.bc == BC_SHOCK) {  // the injection end in cells from nxgs, split into cell + FP32 fraction
    const double xe = shock_xend3(c, c->u0) * d.ph.d_delx - (double)d.g.nxgs;
    const double fl = std::floor(xe);
    c->mk.xend_cell = (int)fl;
    c->mk.xend_frac = (float)(xe - fl);
    if (c->mk.xend_frac >= 1.f) {
      c->mk.xend_frac = 0.f;
      c->mk.xend_cell += 1;
    }
    c->mk.u0 = (float)c->u0;
  }
  mix3_push(d, c->mk, c->tmap, c->pusher == WPIC_PUSH_VAY, c->stream);
  // the arrivals join their columns right away, so the particle state is whole again before the
  // field solve (which does not read particles) can return an error
  mix3_arrive(d, c->stream);
  CK3(cudaMemcpyAsync(c->h_grow, d.m.grow, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  mix3_fix(d, c->stream);
  curre_fold3d(d, c->stream);
  fast::gkl3d(d, c->stream);
  int st = do_cg3(c);
  if (st) return st;
  dfield_ghost3d(d, c->stream);
  fast::efield3d(d, c->stream);
  dfield_ghost3d(d, c->stream);
  uf_add3d(d, c->stream);
  // the CG's host checks synchronised the stream, so the grow flag of this step is in h_grow
  if (*c->h_grow) return mix3_grow(c);
  return WPIC_OK;
}

double shock_xend3(const wpic_ctx3d* c, double u0) {
  return shock_xend_value(c->d.g.nxgs + c->d.g.wx1, c->d.ph.delx, u0, c->d.ph.c, c->d.ph.delt);
}

int one_step3(wpic_ctx3d* c) {
  if (c->mixed) return mixed_step3(c);
  if (c->pusher == WPIC_PUSH_VAY) FP3(push_vay3d, c->d, c->stream);
  else FP3(push3d, c->d, c->stream);
  // the reconnection driver reflects at the walls before the field solve
  // (3d/proj/reconnection/app.f90:103-108), the shock driver applies its injection boundary
  // there and has no particle_x (3d/proj/shock/app.f90:112-117), the periodic one wraps after it
  const int bc = c->d.ph.bc;
  if (bc == BC_RECONNECTION) particle_x3d(c->d, c->d.B, c->stream);
  if (bc == BC_SHOCK) injection3d(c->d, c->d.B, c->u0, shock_xend3(c, c->u0), c->stream);
  int st = do_field3(c);
  if (st) return st;
  if (bc == BC_PERIODIC) particle_x3d(c->d, c->d.B, c->stream);
  do_migrate_sort3(c);
  return WPIC_OK;
}

int put_field3(wpic_ctx3d* c, const double* ref, double* dst, int ncomp) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (!ref) return WPIC_BAD_ARGUMENT;
  const size_t n = (size_t)ncomp * c->d.g.fvol;
  int st = ensure_staging3(c, n * sizeof(double));
  if (st) return st;
  CK3(cudaMemcpyAsync(c->staging, ref, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  field_ref_to_soa(c->staging, dst, ncomp, (int)c->d.g.fvol, c->stream);
  return finish3(c);
}

int get_field3(wpic_ctx3d* c, double* ref, const double* src, int ncomp) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (!ref) return WPIC_BAD_ARGUMENT;
  const size_t n = (size_t)ncomp * c->d.g.fvol;
  int st = ensure_staging3(c, n * sizeof(double));
  if (st) return st;
  field_soa_to_ref(src, c->staging, ncomp, (int)c->d.g.fvol, c->stream);
  CK3(cudaMemcpyAsync(ref, c->staging, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  return finish3(c);
}

}  // namespace

extern "C" {

int wpic3d_init(wpic_ctx3d** out, const wpic_params3d* p, void* cuda_stream) {
  if (!out || !p) return WPIC_BAD_ARGUMENT;
  *out = nullptr;
  const int nx = p->nxge - p->nxgs + 1, ny = p->nyge - p->nygs + 1, nz = p->nzge - p->nzgs + 1;
  if (p->ndim != 7 || p->nsp < 1 || p->nsp > 2 || nx < 4 || ny < 4 || nz < 4 || p->np < 1) return WPIC_BAD_ARGUMENT;
  if (p->nys != p->nygs || p->nye != p->nyge || p->nzs != p->nzgs || p->nze != p->nzge) return WPIC_BAD_ARGUMENT;
  if (!(p->delx > 0) || !(p->delt > 0) || !(p->c > 0)) return WPIC_BAD_ARGUMENT;
  if (p->precision != WPIC_FP64 && p->precision != WPIC_FP64_EXACT && p->precision != WPIC_MIXED)
    return WPIC_BAD_ARGUMENT;
  if (p->precision == WPIC_MIXED && !mix3_shape_ok(nx, ny, nz)) return WPIC_BAD_ARGUMENT;
  if (p->bc_kind != WPIC_BC_PERIODIC && p->bc_kind != WPIC_BC_RECONNECTION && p->bc_kind != WPIC_BC_SHOCK)
    return WPIC_BAD_ARGUMENT;
  if (p->bc_kind != WPIC_BC_PERIODIC && nx < 6) return WPIC_BAD_ARGUMENT;
  if ((double)nx * ny * nz > 2.0e9 || (double)p->nsp * ny * nz * p->np >= 2147483647.0) return WPIC_BAD_ARGUMENT;
  wpic_ctx3d* c = new wpic_ctx3d();
  c->prm = *p;
  Dev3D& d = c->d;
  d.g.nx = nx;
  d.g.ny = ny;
  d.g.nz = nz;
  d.g.nxgs = p->nxgs;
  d.g.nygs = p->nygs;
  d.g.nzgs = p->nzgs;
  d.g.wx0 = 0;
  d.g.wx1 = nx - 1;
  d.g.fp = nx + 4;
  d.g.fplane = (size_t)(nx + 4) * (ny + 4);
  d.g.fvol = d.g.fplane * (nz + 4);
  d.g.ncell = (size_t)nx * ny * nz;
  Phys& ph = d.ph;
  ph.delx = p->delx;
  ph.delt = p->delt;
  ph.c = p->c;
  ph.gfac = p->gfac;
  ph.nsp = p->nsp;
  ph.bc = p->bc_kind == WPIC_BC_RECONNECTION ? BC_RECONNECTION : p->bc_kind == WPIC_BC_SHOCK ? BC_SHOCK : BC_PERIODIC;
  for (int k = 0; k < 2; ++k) {
    ph.q[k] = k < p->nsp ? p->q[k] : 0.0;
    ph.r[k] = k < p->nsp ? p->r[k] : 1.0;
  }
  // field__init constants (3d/common/field.f90:57-63), same operation order
  ph.pi = 4.0 * std::atan(1.0);
  ph.f1 = p->c * p->delt / p->delx;
  ph.f2 = p->gfac * ph.f1 * ph.f1;
  ph.f3 = 4.0 * ph.pi * p->delx / p->c;
  const double t = p->delx / (p->c * p->delt * p->gfac);
  ph.f4 = 6.0 + t * t;
  ph.f5 = t * t;
  ph.p_d_delx = 1.0 / p->delx;
  ph.d_delx = 1.0 / p->delx;
  ph.d_delt = 1.0 / p->delt;
  d.cap = p->device_cap > 0 ? p->device_cap : p->np;
  d.nrow = p->nsp * ny * nz;
  c->mixed = p->precision == WPIC_MIXED;
  if (c->mixed) {
    // FP32 constants of the split-position step, rounded once (the FP64 expressions of
    // 3d/common/particle.f90:106-108 and 3d/common/field.f90:226)
    Mix3Const& k = c->mk;
    double vmax = 0.0;
    for (int s = 0; s < 2; ++s) {
      const bool on = s < p->nsp;
      k.fac1[s] = on ? (float)(p->q[s] / p->r[s] * 0.5 * p->delt) : 0.f;
      k.fac2[s] = on ? (float)(p->q[s] * p->delt / p->r[s]) : 0.f;
      k.qdd[s] = on ? (float)(p->q[s] * p->delx * (1.0 / p->delt)) : 0.f;
      if (on) vmax = std::max(vmax, std::fabs(p->q[s] * p->delx / p->delt));
    }
    k.dtdx = (float)(p->delt / p->delx);
    k.c = (float)p->c;
    k.ic2 = (float)(1.0 / (p->c * p->c));
    // a contribution to one node is at most |q| dx / dt (the Esirkepov weights are at most 1)
    c->mix_vmax = std::max(vmax, 1e-300) * (1.0 + 1e-6);
    Mix3D& m = d.m;
    m.ntx = nx / M3_TX;
    m.nty = ny / M3_TY;
    m.ntz = nz / M3_TZ;
    m.ntile = m.ntx * m.nty * m.ntz;
    m.nbin = m.ntile * p->nsp;
  }
  d.nred = (int)std::min<size_t>(1216, (d.g.ncell + CG_THREADS_HOST - 1) / CG_THREADS_HOST);
  if (d.nred < 1) d.nred = 1;
  d.ite_max = 100;
  if (cuda_stream) {
    c->stream = (cudaStream_t)cuda_stream;
  } else {
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete c;
      return WPIC_CUDA_ERROR;
    }
    c->own_stream = true;
  }
  // the mixed path keeps its particles in the bins: no FP64 particle arrays or migration scratch
  const size_t slots = c->mixed ? 0 : (size_t)d.nrow * d.cap;
  int st = WPIC_OK;
  do {
    if (!c->mixed && ((st = alloc_parts3(c, &d.A, slots)) || (st = alloc_parts3(c, &d.B, slots)))) break;
    if ((st = dalloc3(c, &d.cc, (size_t)d.nrow * (nx + 1))) || (st = dalloc3(c, &d.np2, d.nrow)) ||
        (st = dalloc3(c, &d.np2new, d.nrow)))
      break;
    if ((st = dalloc3(c, &d.uf, 6 * d.g.fvol)) || (st = dalloc3(c, &d.df, 6 * d.g.fvol)) ||
        (st = dalloc3(c, &d.uj, 3 * d.g.fvol)) || (st = dalloc3(c, &d.gkl, 3 * d.g.ncell)))
      break;
    if (c->mixed) {
      Mix3D& m = d.m;
      if ((st = dalloc3(c, &m.boff, (size_t)m.nbin)) || (st = dalloc3(c, &m.bdep, (size_t)m.nbin)) ||
          (st = dalloc3(c, &m.cnt, (size_t)m.nbin * M3_TC)) || (st = dalloc3(c, &m.ccnt, (size_t)m.nbin * M3_TC)) ||
          (st = dalloc3(c, &m.acnt, (size_t)m.nbin * M3_TC)) || (st = dalloc3(c, &m.bneed, (size_t)m.nbin)) ||
          (st = dalloc3(c, &m.grow, 1)) || (st = dalloc3(c, &m.ujx, 3 * d.g.fvol)))
        break;
      if (cudaMallocHost(&c->h_grow, sizeof(int)) != cudaSuccess) { st = WPIC_CUDA_ERROR; break; }
      *c->h_grow = 0;
      if (mix3_setup(d, c->tmap) != 0) { st = WPIC_CUDA_ERROR; break; }
      // an empty layout of shallow columns: wpic3d_put_particles and wpic3d_load_weibel lay the
      // bins out for the particles they bring
      if ((st = mix3_set_layout(c, std::vector<int>(m.nbin, 8), false))) break;
    } else if ((st = dalloc3(c, &d.cellJ, (size_t)375 * d.g.ncell))) {
      break;
    }
    if ((st = dalloc3(c, &d.phi, 3 * d.g.ncell)) || (st = dalloc3(c, &d.p, 3 * d.g.ncell)) ||
        (st = dalloc3(c, &d.r, 3 * d.g.ncell)) || (st = dalloc3(c, &d.ap, 3 * d.g.ncell)) ||
        (st = dalloc3(c, &d.b, 3 * d.g.ncell)))
      break;
    if ((st = dalloc3(c, &d.partials, (size_t)3 * d.nred * 2)) || (st = dalloc3(c, &d.cg, 3)) ||
        (st = dalloc3(c, &d.err, 1)) || (st = dalloc3(c, &d.red_out, 8)))
      break;
    if (!c->mixed &&
        ((st = dalloc3(c, &d.mig, slots)) || (st = dalloc3(c, &d.glist, slots)) ||
         (st = dalloc3(c, &d.gcnt, (size_t)d.nrow * 8)) || (st = dalloc3(c, &d.goff, (size_t)d.nrow * 8)) ||
         (st = dalloc3(c, &d.tlist, slots)) || (st = dalloc3(c, &d.slist, slots)) || (st = dalloc3(c, &d.map, slots))))
      break;
    if (cudaMallocHost(&c->h_cg, 3 * sizeof(CGState)) != cudaSuccess) { st = WPIC_CUDA_ERROR; break; }
    if (cudaMallocHost(&c->h_err, sizeof(int)) != cudaSuccess) { st = WPIC_CUDA_ERROR; break; }
    *c->h_err = 0;
    st = finish3(c);
  } while (false);
  if (st) {
    wpic3d_finalize(c);
    return st;
  }
  *out = c;
  return WPIC_OK;
}

int wpic3d_finalize(wpic_ctx3d* c) {
  if (!c) return WPIC_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (void* p : c->allocs) cudaFree(p);
  if (c->staging) cudaFree(c->staging);
  if (c->mixP) cudaFree(c->mixP);
  if (c->mixK) cudaFree(c->mixK);
  if (c->h_grow) cudaFreeHost(c->h_grow);
  if (c->h_cg) cudaFreeHost(c->h_cg);
  if (c->h_err) cudaFreeHost(c->h_err);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return WPIC_OK;
}

int wpic3d_put_particles(wpic_ctx3d* c, int which, const double* up, const int* np2, const int* cumcnt) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (!up || !np2 || (which == 0 && !cumcnt) || (which != 0 && which != 1)) return WPIC_BAD_ARGUMENT;
  Dev3D& d = c->d;
  const int nx = d.g.nx, ndim = c->prm.ndim, nph = c->prm.np;
  for (int r = 0; r < d.nrow; ++r) {
    if (np2[r] < 0 || np2[r] > d.cap || np2[r] > nph) return WPIC_CAPACITY;
    if (which == 0) {
      const int* cc = cumcnt + (size_t)r * (nx + 1);
      if (cc[0] != 0 || cc[nx] != np2[r]) return WPIC_BAD_ARGUMENT;
      for (int i = 0; i < nx; ++i)
        if (cc[i + 1] < cc[i]) return WPIC_BAD_ARGUMENT;
    }
  }
  if (c->mixed && which == 1) {
    // the unsorted state of the restart path (io__input's up, before sort__bucket; the rows
    // are right, the order within a row is not): each row is bucket-sorted on the host by its
    // x cell i = int(x) as sort__bucket does (3d/common/sort.f90:40-88), stably, and put as the
    // sorted state, which is all a mixed context keeps
    std::vector<double> sorted((size_t)d.nrow * ndim * nph);
    std::vector<int> cc((size_t)d.nrow * (nx + 1));
    std::vector<int> cell(nph);
    for (int r = 0; r < d.nrow; ++r) {
      const double* row = up + (size_t)r * ndim * nph;
      int* crow = cc.data() + (size_t)r * (nx + 1);
      std::fill(crow, crow + nx + 1, 0);
      for (int q = 0; q < np2[r]; ++q) {
        const double x = row[(size_t)q * ndim];
        const int i = (x > -2147483648.0 && x < 2147483647.0) ? (int)x - d.g.nxgs : -1;
        if (i < 0 || i >= nx) return WPIC_OUT_OF_RANGE;
        cell[q] = i;
        ++crow[i + 1];
      }
      for (int i = 0; i < nx; ++i) crow[i + 1] += crow[i];
      std::vector<int> next(crow, crow + nx);
      double* out = sorted.data() + (size_t)r * ndim * nph;
      for (int q = 0; q < np2[r]; ++q)
        std::copy(row + (size_t)q * ndim, row + (size_t)(q + 1) * ndim, out + (size_t)(next[cell[q]]++) * ndim);
    }
    return wpic3d_put_particles(c, 0, sorted.data(), np2, cc.data());
  }
  CK3(cudaMemcpyAsync(d.np2, np2, sizeof(int) * d.nrow, cudaMemcpyHostToDevice, c->stream));
  if (which == 0)
    CK3(cudaMemcpyAsync(d.cc, cumcnt, sizeof(int) * (size_t)d.nrow * (nx + 1), cudaMemcpyHostToDevice, c->stream));
  const size_t row_bytes = (size_t)ndim * nph * sizeof(double);
  if (c->mixed) {
    // lay the bins out for these particles unless every bin already has the room: each bin's
    // depth from its fullest cell, kept while every bin keeps 40 % of its depth free
    Mix3D& m = d.m;
    mix3_binmax(d, c->stream);
    std::vector<int> mx(m.nbin);
    CK3(cudaMemcpyAsync(mx.data(), m.bneed, sizeof(int) * m.nbin, cudaMemcpyDeviceToHost, c->stream));
    CK3(cudaStreamSynchronize(c->stream));
    const double cdx = c->prm.c * c->prm.delt / c->prm.delx;
    std::vector<int> dep(m.nbin);
    bool fits = (int)c->h_dep.size() == m.nbin;
    for (int b = 0; b < m.nbin; ++b) {
      dep[b] = mix3_initial_depth(mx[b], cdx);
      if (fits && 5LL * mx[b] > 3LL * c->h_dep[b]) fits = false;
    }
    int st = fits ? WPIC_OK : mix3_set_layout(c, dep, false);
    if (st) return st;
    CK3(cudaMemsetAsync(m.acnt, 0, sizeof(int) * (size_t)m.nbin * M3_TC, c->stream));
    // one chunk = the 4 ny rows of species isp and z layers 4 tz .. 4 tz + 3 (contiguous in up)
    const size_t chunk_rows = (size_t)M3_TZ * d.g.ny;
    if ((st = ensure_staging3(c, chunk_rows * row_bytes))) return st;
    for (int isp = 0; isp < c->prm.nsp; ++isp)
      for (int tz = 0; tz < m.ntz; ++tz) {
        const size_t r0 = ((size_t)isp * d.g.nz + (size_t)tz * M3_TZ) * d.g.ny;
        CK3(cudaMemcpyAsync(c->staging, up + r0 * ndim * nph, chunk_rows * row_bytes, cudaMemcpyHostToDevice,
                            c->stream));
        mix3_put(d, c->staging, ndim, nph, isp, tz, c->stream);
      }
    return finish3(c);
  }
  size_t rows_per = ((size_t)1 << 30) / row_bytes;
  if (rows_per < 1) rows_per = 1;
  if (rows_per > (size_t)d.nrow) rows_per = d.nrow;
  int st = ensure_staging3(c, rows_per * row_bytes);
  if (st) return st;
  const Parts3D& P = which == 0 ? d.A : d.B;
  for (int r0 = 0; r0 < d.nrow; r0 += (int)rows_per) {
    const int nr = (int)std::min<size_t>(rows_per, (size_t)(d.nrow - r0));
    CK3(cudaMemcpyAsync(c->staging, up + (size_t)r0 * ndim * nph, nr * row_bytes, cudaMemcpyHostToDevice, c->stream));
    aos_to_soa3d(d, c->staging, ndim, nph, r0, nr, P, c->stream);
  }
  return finish3(c);
}

int wpic3d_get_particles(wpic_ctx3d* c, int which, double* up, int* np2, int* cumcnt) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (!up || (which != 0 && which != 1)) return WPIC_BAD_ARGUMENT;
  Dev3D& d = c->d;
  const int nx = d.g.nx, ndim = c->prm.ndim, nph = c->prm.np;
  if (c->mixed) {
    if (which != 0) return WPIC_BAD_ARGUMENT;
    mix3_count_rows(d, c->stream);
    std::vector<int> h(d.nrow);
    CK3(cudaMemcpyAsync(h.data(), d.np2, sizeof(int) * d.nrow, cudaMemcpyDeviceToHost, c->stream));
    if (cumcnt)
      CK3(cudaMemcpyAsync(cumcnt, d.cc, sizeof(int) * (size_t)d.nrow * (nx + 1), cudaMemcpyDeviceToHost, c->stream));
    CK3(cudaStreamSynchronize(c->stream));
    for (int r = 0; r < d.nrow; ++r)
      if (h[r] > nph) return WPIC_CAPACITY;
    if (np2) std::copy(h.begin(), h.end(), np2);
    const size_t row_bytes = (size_t)ndim * nph * sizeof(double);
    const size_t chunk_rows = (size_t)M3_TZ * d.g.ny;
    int st = ensure_staging3(c, chunk_rows * row_bytes);
    if (st) return st;
    for (int isp = 0; isp < c->prm.nsp; ++isp)
      for (int tz = 0; tz < d.m.ntz; ++tz) {
        const size_t r0 = ((size_t)isp * d.g.nz + (size_t)tz * M3_TZ) * d.g.ny;
        CK3(cudaMemsetAsync(c->staging, 0, chunk_rows * row_bytes, c->stream));
        mix3_get(d, c->staging, ndim, nph, isp, tz, c->stream);
        CK3(cudaMemcpyAsync(up + r0 * ndim * nph, c->staging, chunk_rows * row_bytes, cudaMemcpyDeviceToHost,
                            c->stream));
      }
    return finish3(c);
  }
  if (np2) CK3(cudaMemcpyAsync(np2, d.np2, sizeof(int) * d.nrow, cudaMemcpyDeviceToHost, c->stream));
  if (cumcnt && which == 0)
    CK3(cudaMemcpyAsync(cumcnt, d.cc, sizeof(int) * (size_t)d.nrow * (nx + 1), cudaMemcpyDeviceToHost, c->stream));
  const size_t row_bytes = (size_t)ndim * nph * sizeof(double);
  size_t rows_per = ((size_t)1 << 30) / row_bytes;
  if (rows_per < 1) rows_per = 1;
  if (rows_per > (size_t)d.nrow) rows_per = d.nrow;
  int st = ensure_staging3(c, rows_per * row_bytes);
  if (st) return st;
  const Parts3D& P = which == 0 ? d.A : d.B;
  for (int r0 = 0; r0 < d.nrow; r0 += (int)rows_per) {
    const int nr = (int)std::min<size_t>(rows_per, (size_t)(d.nrow - r0));
    CK3(cudaMemsetAsync(c->staging, 0, nr * row_bytes, c->stream));
    soa_to_aos3d(d, c->staging, ndim, nph, r0, nr, P, c->stream);
    CK3(cudaMemcpyAsync(up + (size_t)r0 * ndim * nph, c->staging, nr * row_bytes, cudaMemcpyDeviceToHost, c->stream));
  }
  return finish3(c);
}

int wpic3d_put_fields(wpic_ctx3d* c, const double* uf) { return c ? put_field3(c, uf, c->d.uf, 6) : WPIC_NOT_INITIALISED; }
int wpic3d_get_fields(wpic_ctx3d* c, double* uf) { return c ? get_field3(c, uf, c->d.uf, 6) : WPIC_NOT_INITIALISED; }
int wpic3d_put_df(wpic_ctx3d* c, const double* df) { return c ? put_field3(c, df, c->d.df, 6) : WPIC_NOT_INITIALISED; }
int wpic3d_get_df(wpic_ctx3d* c, double* df) { return c ? get_field3(c, df, c->d.df, 6) : WPIC_NOT_INITIALISED; }
int wpic3d_get_uj(wpic_ctx3d* c, double* uj) { return c ? get_field3(c, uj, c->d.uj, 3) : WPIC_NOT_INITIALISED; }

namespace {
// The staged calls on a mixed context (the 3D counterpart of the 2D mapping): particle__solv
// asks for the push, field__fdtd_i runs the fused mixed step (push, deposit, x boundary,
// cell-leavers into their columns, field solve), particle_x, particle_yz and sort__bucket find
// their work done; the shock driver's injection call between the push and the field solve
// sets the step's u0.
int mix3_request_push(wpic_ctx3d* c, int pusher) {
  if (c->mix_pending) return WPIC_BAD_ARGUMENT;  // a second push before the field solve
  c->mix_pending = true;
  c->mix_pending_pusher = pusher;
  return WPIC_OK;
}

int mix3_run_requested(wpic_ctx3d* c) {
  if (!c->mix_pending) return WPIC_BAD_ARGUMENT;  // the field solve cannot run without its push
  c->mix_pending = false;
  const int saved = c->pusher;
  c->pusher = c->mix_pending_pusher;
  int st = one_step3(c);
  c->pusher = saved;
  const int st2 = finish3(c);
  return st ? st : st2;
}
}  // namespace

int wpic3d_particle_solv(wpic_ctx3d* c) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mixed) return mix3_request_push(c, WPIC_PUSH_BORIS);
  FP3(push3d, c->d, c->stream);
  return finish3(c);
}

int wpic3d_particle_solv_vay(wpic_ctx3d* c) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mixed) return mix3_request_push(c, WPIC_PUSH_VAY);
  FP3(push_vay3d, c->d, c->stream);
  return finish3(c);
}

int wpic3d_set_pusher(wpic_ctx3d* c, int pusher) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (pusher != WPIC_PUSH_BORIS && pusher != WPIC_PUSH_VAY) return WPIC_BAD_ARGUMENT;
  c->pusher = pusher;
  return WPIC_OK;
}

int wpic3d_field_fdtd_i(wpic_ctx3d* c) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mixed) return mix3_run_requested(c);
  int st = do_field3(c);
  if (st) return st;
  return finish3(c);
}

// ele_cur + bc__curre of field__fdtd_i (3d/common/field.f90:129-130), for parity checks
int wpic3d_ele_cur(wpic_ctx3d* c) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mixed) return WPIC_BAD_ARGUMENT;  // the mixed path runs fused steps only
  FP3(deposit3d, c->d, c->stream);
  curre_fold3d(c->d, c->stream);
  return finish3(c);
}

int wpic3d_bc_particle_x(wpic_ctx3d* c) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->d.ph.bc == BC_SHOCK) return WPIC_BAD_ARGUMENT;  // boundary_shock has no particle_x
  if (c->mixed) return WPIC_OK;  // inside the mixed step, before or after its field solve
  particle_x3d(c->d, c->d.B, c->stream);
  return finish3(c);
}

int wpic3d_set_window(wpic_ctx3d* c, int nxs, int nxe) {
  if (!c) return WPIC_NOT_INITIALISED;
  const int nxge = c->d.g.nxgs + c->d.g.nx - 1;
  if (nxs < c->d.g.nxgs || nxe > nxge || nxe - nxs < 3) return WPIC_BAD_ARGUMENT;
  const bool full = nxs == c->d.g.nxgs && nxe == nxge;
  if (!full && c->d.ph.bc != BC_SHOCK) return WPIC_BAD_ARGUMENT;
  c->d.g.wx0 = nxs - c->d.g.nxgs;
  c->d.g.wx1 = nxe - c->d.g.nxgs;
  return WPIC_OK;
}

int wpic3d_set_injection(wpic_ctx3d* c, double u0) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (!(u0 == u0)) return WPIC_BAD_ARGUMENT;
  c->u0 = u0;
  return WPIC_OK;
}

int wpic3d_bc_injection(wpic_ctx3d* c, double u0) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->d.ph.bc != BC_SHOCK || !(u0 == u0)) return WPIC_BAD_ARGUMENT;
  if (c->mixed) {  // between the requested push and the field solve: the step's u0
    if (!c->mix_pending) return WPIC_BAD_ARGUMENT;
    c->u0 = u0;
    return WPIC_OK;
  }
  injection3d(c->d, c->d.B, u0, shock_xend3(c, u0), c->stream);
  return finish3(c);
}

// bc__particle_yz on gp (B) in place: the post-migration order is gathered through map = slist
int wpic3d_bc_particle_yz(wpic_ctx3d* c) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mixed) return c->mix_pending ? WPIC_BAD_ARGUMENT : WPIC_OK;  // done by the mixed step
  Dev3D& d = c->d;
  migrate_scan3d(d, d.B, c->stream);
  migrate_plan3d(d, c->stream);
  // gather B -> A by slist, then copy back into B (A is the sorted state, rebuilt by sort_bucket)
  gather3d(d, d.B, d.A, d.slist, d.np2new, c->stream);
  const size_t slots = (size_t)d.nrow * d.cap;
  CK3(cudaMemcpyAsync(d.B.x, d.A.x, slots * 8, cudaMemcpyDeviceToDevice, c->stream));
  CK3(cudaMemcpyAsync(d.B.y, d.A.y, slots * 8, cudaMemcpyDeviceToDevice, c->stream));
  CK3(cudaMemcpyAsync(d.B.z, d.A.z, slots * 8, cudaMemcpyDeviceToDevice, c->stream));
  CK3(cudaMemcpyAsync(d.B.ux, d.A.ux, slots * 8, cudaMemcpyDeviceToDevice, c->stream));
  CK3(cudaMemcpyAsync(d.B.uy, d.A.uy, slots * 8, cudaMemcpyDeviceToDevice, c->stream));
  CK3(cudaMemcpyAsync(d.B.uz, d.A.uz, slots * 8, cudaMemcpyDeviceToDevice, c->stream));
  CK3(cudaMemcpyAsync(d.B.id, d.A.id, slots * 8, cudaMemcpyDeviceToDevice, c->stream));
  CK3(cudaMemcpyAsync(d.np2, d.np2new, sizeof(int) * d.nrow, cudaMemcpyDeviceToDevice, c->stream));
  return finish3(c);
}

// sort__bucket: gp (B) -> up (A) with cumcnt
int wpic3d_sort_bucket(wpic_ctx3d* c) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mixed) return c->mix_pending ? WPIC_BAD_ARGUMENT : WPIC_OK;  // done by the mixed step
  Dev3D& d = c->d;
  sort_rank3d(d, d.B, nullptr, c->stream);
  gather3d(d, d.B, d.A, d.map, d.np2, c->stream);
  return finish3(c);
}

int wpic3d_step(wpic_ctx3d* c, int nsteps) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mix_pending) return WPIC_BAD_ARGUMENT;  // a requested push waits for field__fdtd_i
  for (int it = 0; it < nsteps; ++it) {
    int st = one_step3(c);
    if (st) return st;
    st = finish3(c);
    if (st) return st;
  }
  return WPIC_OK;
}

int wpic3d_energy(wpic_ctx3d* c, double* out) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (!out) return WPIC_BAD_ARGUMENT;
  if (c->mixed) mix3_energy(c->d, c->stream);
  else FP3(energy3d, c->d, c->stream);
  double h[4];
  CK3(cudaMemcpyAsync(h, c->d.red_out, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  int st = finish3(c);
  if (st) return st;
  const int nsp = c->prm.nsp;
  for (int k = 0; k < nsp; ++k) out[k] = h[k];
  out[nsp] = h[2];
  out[nsp + 1] = h[3];
  return WPIC_OK;
}

namespace {
size_t mom_count3(const wpic_ctx3d* c) {
  return 7 * (size_t)(c->d.g.nx + 2) * (c->d.g.ny + 2) * (c->d.g.nz + 2) * c->d.ph.nsp;
}
int ensure_mom3(wpic_ctx3d* c) {
  if (c->mom) return WPIC_OK;
  return dalloc3(c, &c->mom, mom_count3(c));
}
int copy_mom3(wpic_ctx3d* c, double* out) {
  if (!out) return WPIC_OK;
  CK3(cudaMemcpyAsync(out, c->mom, mom_count3(c) * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  return WPIC_OK;
}
}  // namespace

// mixed context: mom_calc__nvt (from gp) computes the folded moments with the FP32 half-step
// push, mom_calc__accl and bc__mom have nothing left to do
int wpic3d_mom_calc_accl(wpic_ctx3d* c) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mixed) return c->mix_pending ? WPIC_BAD_ARGUMENT : WPIC_OK;
  FP3(mom_accl3d, c->d, c->stream);
  return finish3(c);
}

int wpic3d_mom_calc_nvt(wpic_ctx3d* c, int from_gp) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (from_gp != 0 && from_gp != 1) return WPIC_BAD_ARGUMENT;
  if (c->mixed && (from_gp != 1 || c->mix_pending)) return WPIC_BAD_ARGUMENT;
  int st = ensure_mom3(c);
  if (st) return st;
  if (c->mixed) mix3_moments(c->d, c->mk, c->mom, c->stream);
  else FP3(mom_nvt3d, c->d, from_gp ? c->d.B : c->d.A, c->mom, c->stream);
  return finish3(c);
}

int wpic3d_bc_mom(wpic_ctx3d* c) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (!c->mom) return WPIC_BAD_ARGUMENT;
  if (c->mixed) return WPIC_OK;  // the mixed moments come folded
  bc_mom3d(c->d, c->mom, c->stream);
  return finish3(c);
}

int wpic3d_get_mom(wpic_ctx3d* c, double* mom) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (!c->mom || !mom) return WPIC_BAD_ARGUMENT;
  int st = copy_mom3(c, mom);
  if (st) return st;
  return finish3(c);
}

int wpic3d_moments(wpic_ctx3d* c, double* mom) {
  if (!c) return WPIC_NOT_INITIALISED;
  int st = ensure_mom3(c);
  if (st) return st;
  if (c->mixed) {
    mix3_moments(c->d, c->mk, c->mom, c->stream);  // from the bins: no gp is written
  } else {
    FP3(mom_accl3d, c->d, c->stream);
    FP3(mom_nvt3d, c->d, c->d.B, c->mom, c->stream);
    bc_mom3d(c->d, c->mom, c->stream);
  }
  if ((st = copy_mom3(c, mom))) return st;
  return finish3(c);
}

int wpic3d_cg_control(wpic_ctx3d* c, const int* fixed3, int ite_max) {
  if (!c) return WPIC_NOT_INITIALISED;
  for (int l = 0; l < 3; ++l) c->cg_fixed[l] = fixed3 ? fixed3[l] : -1;
  c->d.ite_max = ite_max > 0 ? ite_max : 100;
  return WPIC_OK;
}

int wpic3d_cg_iters(wpic_ctx3d* c, int* out3) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (!out3) return WPIC_BAD_ARGUMENT;
  for (int l = 0; l < 3; ++l) out3[l] = c->cg_iters[l];
  return WPIC_OK;
}

int wpic3d_load_weibel(wpic_ctx3d* c, int ppc, uint64_t seed, double drift, int drift_axis, double u_thi,
                       double u_the) {
  if (!c) return WPIC_NOT_INITIALISED;
  Dev3D& d = c->d;
  if (drift_axis < 0 || drift_axis > 2 || ppc < 1) return WPIC_BAD_ARGUMENT;
  if (c->mixed) {
    const int dep = mix3_initial_depth(ppc, c->prm.c * c->prm.delt / c->prm.delx);
    int st = mix3_set_layout(c, std::vector<int>(d.m.nbin, dep), false);
    if (st) return st;
    CK3(cudaMemsetAsync(d.m.acnt, 0, sizeof(int) * (size_t)d.m.nbin * M3_TC, c->stream));
    mix3_load_weibel(d, ppc, seed, drift, drift_axis, u_thi, u_the, c->stream);
  } else {
    if ((long long)ppc * d.g.nx > d.cap) return WPIC_CAPACITY;
    load_weibel3d_ppc(d, ppc, seed, drift, drift_axis, u_thi, u_the, c->stream);
  }
  CK3(cudaMemsetAsync(d.uf, 0, 6 * d.g.fvol * sizeof(double), c->stream));
  CK3(cudaMemsetAsync(d.df, 0, 6 * d.g.fvol * sizeof(double), c->stream));
  CK3(cudaMemsetAsync(d.uj, 0, 3 * d.g.fvol * sizeof(double), c->stream));
  return finish3(c);
}

long long wpic3d_num_particles(wpic_ctx3d* c) {
  if (!c) return -1;
  const bool mx = c->mixed;
  std::vector<int> h(mx ? (size_t)c->d.m.nbin * M3_TC : (size_t)c->d.nrow);
  if (cudaMemcpyAsync(h.data(), mx ? c->d.m.cnt : c->d.np2, sizeof(int) * h.size(), cudaMemcpyDeviceToHost,
                      c->stream) != cudaSuccess)
    return -1;
  cudaStreamSynchronize(c->stream);
  long long n = 0;
  for (int v : h) n += v;
  return n;
}

int wpic3d_synchronize(wpic_ctx3d* c) { return c ? finish3(c) : WPIC_NOT_INITIALISED; }

}  // extern "C"
