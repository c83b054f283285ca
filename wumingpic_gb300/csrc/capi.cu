// C ABI of the library (declared in include/wumingpic_gb300.h): context
// creation, device memory, reference-layout state exchange, and the host-side
// sequencing of the kernels of one time step.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "wumingpic_gb300.h"
#include "wpic_internal.h"

using namespace wpic;

namespace {

enum Stage { SG_PUSH, SG_DEPOSIT, SG_JREDUCE, SG_FIELD, SG_CG, SG_PBC, SG_SORT, SG_COUNT };
const char* kStageNames[SG_COUNT] = {"push", "deposit", "current_reduce", "field", "cg", "particle_bc", "sort"};

constexpr int CG_CHECK_EVERY = 4;  // CG iterations enqueued between host checks of the active flags

}  // namespace

struct wpic_ctx {
  wpic_params prm;
  Dev2D d;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  CGState* h_cg = nullptr;  // pinned mirror of the CG states
  int* h_err = nullptr;     // pinned mirror of the error word
  int cg_fixed[3] = {-1, -1, -1};
  int cg_pred = 4;  // iterations enqueued before the first host check: the last solve's count
  int cg_iters[3] = {0, 0, 0};
  std::vector<void*> allocs;
  double* staging = nullptr;
  size_t staging_bytes = 0;
  bool have_C = false;
  bool timing = false;
  cudaEvent_t ev0[SG_COUNT], ev1[SG_COUNT];
  bool pending[SG_COUNT] = {};
  double stage_ms[SG_COUNT] = {};
  long long stage_launches[SG_COUNT] = {};
  int sticky_status = WPIC_OK;
  bool mixed = false;
  alignas(128) unsigned char tmap[128];  // CUtensorMap of uf (mixed path TMA loads)
  // mixed path: the particle layers (reallocated when bins grow) and the host copy of the layout
  float* mixP = nullptr;
  std::vector<int> h_dep;
  std::vector<long long> h_off;
  int* h_grow = nullptr;  // pinned mirror of the grow flag
  // mixed path state exchange: a copy stream and two staging buffers used in turn, so that
  // the host link transfers one chunk while the device converts the other
  // two copy streams take alternate rows, so that one copy's setup overlaps the other's transfer
  cudaStream_t xfer[2] = {nullptr, nullptr};
  double* xstg[2] = {nullptr, nullptr};
  size_t xstg_bytes = 0;
  cudaEvent_t ev_copied[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [buffer][copy stream]
  cudaEvent_t ev_used[2] = {nullptr, nullptr};
  std::vector<int> h_np2;
  double mix_vmax = 0.0;  // largest contribution of one particle to one node of the deposit
  int pusher = WPIC_PUSH_BORIS;  // the push of the fused step
  // the drivers' staged calls on a mixed context: particle__solv asks for the push
  // (mix_pending, with its pusher) and field__fdtd_i runs the fused mixed step
  bool mix_pending = false;
  int mix_pending_pusher = WPIC_PUSH_BORIS;
  double* mom = nullptr;         // mom(7, nxgs-1:nxge+1, nys-1:nye+1, nsp), allocated on first use
  double u0 = 0.0;               // shock: upstream four-velocity of the injection boundary
  // adjoint: adjoint particle arrays (sorted-state and pushed slots), field adjoints, the
  // cell-centred fields and their adjoint, and the stored states of the reverse sweep
  struct AdjState {
    Parts64 A;
    int *cc, *np2;
    double *uf, *df;
    // states of a recomputed segment also keep the step's pushed particles and permutation
    Parts64 B{};
    int *map = nullptr, *np2new = nullptr;
    bool has_step = false;
  };
  bool adj_ready = false;
  Parts64 lA{}, lB{};
  double *luf = nullptr, *ldf = nullptr, *luj = nullptr, *lg = nullptr, *tmpc = nullptr, *ltmp = nullptr;
  int* adj_cc = nullptr;  // the step's cell offsets, kept across the sort that gives the permutation
  int adj_nsteps = 0, adj_every = 1;  // the recorded forward run (0: none)
  int adj_fp32 = 0;  // the reverse push and deposit sweeps in FP32 (fields, CG and sums in FP64)
  bool adj_last_kept = false;  // the step states hold the recorded run's last segment
  // the field state (uf, df) before each step j = 1 .. adj_nfield of the recorded run, slot
  // j - 1: a recomputed segment then pushes and sorts only, its fields replayed from here
  // instead of deposited and solved again
  double* adj_fields = nullptr;
  size_t adj_fields_slots = 0;  // states the buffer holds
  int adj_nfield = 0;           // states of the recorded run in it
  bool adj_keep_fields = true;  // wpic_adjoint_keep_fields
  float* adj_f32 = nullptr;     // FP32 copies of lJ / the cell-centred fields for the FP32 sweeps
  // scratch of the adjoint's self-checks, allocated on first use
  double* chk_dots = nullptr;
  Parts64 chk_A0{}, chk_B0{}, chk_vA{}, chk_vB{};
  double *chk_f0 = nullptr, *chk_v = nullptr, *chk_lj = nullptr;
  std::vector<AdjState> adj_states;
};

namespace {

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return WPIC_OK;
  fprintf(stderr, "wumingpic_gb300: CUDA error %s\n", cudaGetErrorString(e));
  return WPIC_CUDA_ERROR;
}

#define CK(call)                                   \
  do {                                             \
    cudaError_t e_ = (call);                       \
    if (e_ != cudaSuccess) return cuda_status(e_); \
  } while (0)

template <typename T>
int dalloc(wpic_ctx* c, T** p, size_t n) {
  void* v = nullptr;
  cudaError_t e = cudaMalloc(&v, n * sizeof(T) + 16);
  if (e != cudaSuccess) return cuda_status(e);
  c->allocs.push_back(v);
  e = cudaMemsetAsync(v, 0, n * sizeof(T) + 16, c->stream);
  if (e != cudaSuccess) return cuda_status(e);
  *p = (T*)v;
  return WPIC_OK;
}

int alloc_parts(wpic_ctx* c, Parts64* P, size_t n) {
  int st;
  if ((st = dalloc(c, &P->x, n))) return st;
  if ((st = dalloc(c, &P->y, n))) return st;
  if ((st = dalloc(c, &P->ux, n))) return st;
  if ((st = dalloc(c, &P->uy, n))) return st;
  if ((st = dalloc(c, &P->uz, n))) return st;
  if ((st = dalloc(c, &P->id, n))) return st;
  return WPIC_OK;
}

void stage_begin(wpic_ctx* c, int s) {
  if (c->timing) cudaEventRecord(c->ev0[s], c->stream);
}
void stage_end(wpic_ctx* c, int s, int launches) {
  c->stage_launches[s] += launches;
  if (c->timing) {
    cudaEventRecord(c->ev1[s], c->stream);
    c->pending[s] = true;
  }
}
// Resolve recorded stage events; call after the stream has been synchronised.
void stage_collect(wpic_ctx* c) {
  if (!c->timing) return;
  for (int s = 0; s < SG_COUNT; ++s)
    if (c->pending[s]) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, c->ev0[s], c->ev1[s]) == cudaSuccess) c->stage_ms[s] += ms;
      c->pending[s] = false;
    }
}

// Synchronise, fold the device error word into a status, clear it.
int finish(wpic_ctx* c) {
  cudaError_t e = cudaMemcpyAsync(c->h_err, c->d.err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e);
  stage_collect(c);
  const int bits = *c->h_err;
  if (bits) cudaMemsetAsync(c->d.err, 0, sizeof(int), c->stream);
  if (bits & EB_STAGING_TIMEOUT) return WPIC_STAGING_TIMEOUT;
  if (bits & EB_MOVED_TOO_FAR) return WPIC_MOVED_TOO_FAR;
  if (bits & EB_OUT_OF_RANGE) return WPIC_OUT_OF_RANGE;
  if (bits & EB_CAPACITY) return WPIC_CAPACITY;
  if (bits & EB_CG) return WPIC_CG_NOT_CONVERGED;
  return WPIC_OK;
}

bool exact_mode(const wpic_ctx* c) { return c->prm.precision == WPIC_FP64_EXACT; }

#define FP(fn, ...)                       \
  do {                                    \
    if (exact_mode(c)) exact::fn(__VA_ARGS__); \
    else fast::fn(__VA_ARGS__);           \
  } while (0)

int ensure_staging(wpic_ctx* c, size_t bytes) {
  if (c->staging_bytes >= bytes) return WPIC_OK;
  if (c->staging) {
    cudaStreamSynchronize(c->stream);
    cudaFree(c->staging);
    c->staging = nullptr;
    c->staging_bytes = 0;
  }
  CK(cudaMalloc(&c->staging, bytes));
  c->staging_bytes = bytes;
  return WPIC_OK;
}

// copy streams, events and two staging buffers of `bytes` each for the mixed state exchange
int ensure_xfer(wpic_ctx* c, size_t bytes) {
  if (!c->xfer[0]) {
    for (int k = 0; k < 2; ++k) {
      CK(cudaStreamCreateWithFlags(&c->xfer[k], cudaStreamNonBlocking));
      for (int q = 0; q < 2; ++q) CK(cudaEventCreateWithFlags(&c->ev_copied[k][q], cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&c->ev_used[k], cudaEventDisableTiming));
    }
  }
  if (c->xstg_bytes < bytes) {
    for (int k = 0; k < 2; ++k) CK(cudaStreamSynchronize(c->xfer[k]));
    CK(cudaStreamSynchronize(c->stream));
    for (int k = 0; k < 2; ++k) {
      if (c->xstg[k]) cudaFree(c->xstg[k]);
      c->xstg[k] = nullptr;
    }
    c->xstg_bytes = 0;
    for (int k = 0; k < 2; ++k) CK(cudaMalloc(&c->xstg[k], bytes));
    c->xstg_bytes = bytes;
  }
  return WPIC_OK;
}

int sync_xfer(wpic_ctx* c) {
  for (int k = 0; k < 2; ++k) CK(cudaStreamSynchronize(c->xfer[k]));
  return WPIC_OK;
}

// ---- the stages of one step ----

void do_push(wpic_ctx* c) {
  stage_begin(c, SG_PUSH);
  if (c->pusher == WPIC_PUSH_VAY) FP(push_vay2d, c->d, c->stream);
  else FP(push2d, c->d, c->stream);
  stage_end(c, SG_PUSH, 1);
}

void do_ele_cur(wpic_ctx* c) {
  stage_begin(c, SG_DEPOSIT);
  FP(deposit2d, c->d, c->stream);  // k_deposit2d + k_jgather2d
  stage_end(c, SG_DEPOSIT, 2);
  stage_begin(c, SG_JREDUCE);
  curre_fold2d(c->d, c->stream);
  stage_end(c, SG_JREDUCE, c->d.ph.bc == BC_PERIODIC ? 2 : 1);
}

int do_cg(wpic_ctx* c) {
  stage_begin(c, SG_CG);
  for (int l = 0; l < 3; ++l) c->h_cg[l].fixed = c->cg_fixed[l];
  // publish the fixed counts; the rest of the state is (re)initialised by the init kernels
  for (int l = 0; l < 3; ++l)
    CK(cudaMemcpyAsync(&c->d.cg[l].fixed, &c->h_cg[l].fixed, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  FP(cg_init2d, c->d, c->stream);
  int launches = 2;
  // The iterations run on device flags (a component that has converged returns at once), so
  // the host only decides when to stop enqueueing: first as many iterations as the last solve
  // took (the field changes little from step to step), then CG_CHECK_EVERY at a time.
  int chunk = c->cg_pred;
  for (int guard = 0; guard < 100000; ++guard) {
    for (int k = 0; k < chunk; ++k) {
      FP(cg_iter_ap2d, c->d, c->stream);
      FP(cg_iter_update2d, c->d, c->stream);
      FP(cg_iter_p2d, c->d, c->stream);
      launches += 6;
    }
    CK(cudaMemcpyAsync(c->h_cg, c->d.cg, 3 * sizeof(CGState), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (!c->h_cg[0].active && !c->h_cg[1].active && !c->h_cg[2].active) break;
    chunk = CG_CHECK_EVERY;
  }
  int most = 1;
  for (int l = 0; l < 3; ++l) {
    c->cg_iters[l] = c->h_cg[l].ite;
    most = std::max(most, c->h_cg[l].ite);
  }
  c->cg_pred = std::min(most, 100);
  FP(cg_store2d, c->d, c->stream);
  stage_end(c, SG_CG, launches + 1);
  return WPIC_OK;
}

int do_field(wpic_ctx* c) {
  do_ele_cur(c);
  stage_begin(c, SG_FIELD);
  FP(gkl2d, c->d, c->stream);
  stage_end(c, SG_FIELD, 1);
  int st = do_cg(c);
  if (st) return st;
  stage_begin(c, SG_FIELD);
  dfield_ghost2d(c->d, c->stream);
  FP(efield2d, c->d, c->stream);
  dfield_ghost2d(c->d, c->stream);
  uf_add2d(c->d, c->stream);
  stage_end(c, SG_FIELD, 6);
  return WPIC_OK;
}

void do_particle_x(wpic_ctx* c) {
  stage_begin(c, SG_PBC);
  particle_x2d(c->d, c->d.B, c->stream);
  stage_end(c, SG_PBC, 1);
}

int ensure_C(wpic_ctx* c) {
  if (c->have_C) return WPIC_OK;
  int st = alloc_parts(c, &c->d.C, (size_t)c->d.nrowjob * c->d.cap);
  if (st) return st;
  c->have_C = true;
  return WPIC_OK;
}

// fused migration + bucket sort: B (post-push, post-x-boundary) -> A sorted; wrapx: the periodic
// particle_x in the same pass over the particles as the first phase of particle_y
void do_migrate_sort(wpic_ctx* c, bool wrapx = false) {
  stage_begin(c, SG_PBC);
  if (wrapx) wrapx_migrate_scan2d(c->d, c->d.B, c->stream);
  else migrate_scan2d(c->d, c->d.B, c->stream);
  migrate_plan2d(c->d, c->stream);
  stage_end(c, SG_PBC, 2);
  stage_begin(c, SG_SORT);
  sort_rank2d(c->d, c->d.B, c->d.slist, c->stream);
  gather2d(c->d, c->d.B, c->d.A, c->d.map, c->d.np2new, c->stream);
  cudaMemcpyAsync(c->d.np2, c->d.np2new, sizeof(int) * c->d.nrowjob, cudaMemcpyDeviceToDevice, c->stream);
  stage_end(c, SG_SORT, 2);
}

// Fixed-point scales of the mixed deposit for columns of at most maxdep slots.  One particle adds
// at most vmax = max(|q| dx/dt, 2 |q| c) to a node; a thread flushes the sum of up to MIX_FLUSH
// particles at once (|v s1| <= 2^21 keeps the magic-number rounding exact), and at most
// 25 * nsp * maxdep particles reach a node in one tile pass (|sum hi| < 2^30).  The current is
// rebuilt every step, so the scales may change with the layout.
int mix_set_scales(wpic_ctx* c, int maxdep) {
  Mix2D& m = c->d.m;
  const double vmax = c->mix_vmax;
  const int nsp = c->prm.nsp;
  double s1 = std::ldexp(1.0, 21) / (MIX_FLUSH * vmax);
  const double lim = std::ldexp(1.0, 30) / (25.0 * nsp * maxdep * vmax);
  if (lim < s1) s1 = lim;
  s1 = std::ldexp(1.0, (int)std::floor(std::log2(s1)));
  // lo plane: each flush adds |lo| <= 2^14; a node takes at most 25 * ceil(nsp * maxdep / MIX_FLUSH) flushes
  const double nflush = 25.0 * std::ceil((double)nsp * maxdep / MIX_FLUSH) + 25.0;
  if (!(s1 > 0.0) || s1 > std::ldexp(1.0, 100) || nflush * 16384.0 >= std::ldexp(1.0, 31)) return WPIC_BAD_ARGUMENT;
  m.fx_s1 = (float)s1;
  m.fx_is1f = (float)(1.0 / s1);
  m.fx_s2 = (float)(s1 * 32768.0);
  m.fx_is1 = 1.0 / s1;
  m.fx_is2 = 1.0 / (s1 * 32768.0);
  return WPIC_OK;
}

// Lays the mixed-path bins out with the given depths (slots per column).  keep = true copies
// the columns of the current layout (counts unchanged); otherwise the new layout starts empty.
int mix_set_layout(wpic_ctx* c, const std::vector<int>& dep, bool keep) {
  Mix2D& m = c->d.m;
  std::vector<long long> off(m.nbin);
  long long layers = 0;
  int maxdep = 1;
  for (int b = 0; b < m.nbin; ++b) {
    if (dep[b] < 1 || dep[b] > MIX_MAX_DEPTH) return WPIC_CAPACITY;
    off[b] = layers;
    layers += dep[b];
    maxdep = std::max(maxdep, dep[b]);
  }
  if (int st = mix_set_scales(c, maxdep)) return st;
  if (!keep && c->mixP) {
    CK(cudaStreamSynchronize(c->stream));
    cudaFree(c->mixP);
    c->mixP = nullptr;
  }
  float* np_ = nullptr;
  CK(cudaMalloc(&np_, (size_t)layers * MIX_PL * sizeof(float)));
  long long* old_off = nullptr;
  const float* old_P = c->mixP;
  if (keep && old_P) {
    // the old offsets stay readable by the copy kernel until it is done
    CK(cudaMalloc(&old_off, sizeof(long long) * m.nbin));
    CK(cudaMemcpyAsync(old_off, m.boff, sizeof(long long) * m.nbin, cudaMemcpyDeviceToDevice, c->stream));
  }
  CK(cudaMemcpyAsync(m.boff, off.data(), sizeof(long long) * m.nbin, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(m.bdep, dep.data(), sizeof(int) * m.nbin, cudaMemcpyHostToDevice, c->stream));
  m.P = np_;
  if (keep && old_P) mix_relayout2d(c->d, old_P, old_off, c->stream);
  CK(cudaStreamSynchronize(c->stream));  // host vectors and the old buffers are released below
  if (old_off) cudaFree(old_off);
  if (keep && old_P) cudaFree(c->mixP);
  c->mixP = np_;
  c->h_dep = dep;
  c->h_off = off;
  return WPIC_OK;
}

// grows the bins whose columns came within 1/8 of full in the last step to 1.5 x their need
int mix_grow(wpic_ctx* c) {
  Mix2D& m = c->d.m;
  std::vector<int> need(m.nbin);
  CK(cudaMemcpyAsync(need.data(), m.bneed, sizeof(int) * m.nbin, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemsetAsync(m.grow, 0, sizeof(int), c->stream));
  CK(cudaStreamSynchronize(c->stream));
  *c->h_grow = 0;
  std::vector<int> dep = c->h_dep;
  bool any = false;
  for (int b = 0; b < m.nbin; ++b)
    if (8LL * need[b] > 7LL * dep[b]) {
      const long long nd = ((long long)std::ceil(1.5 * need[b] + 16.0) + 7) & ~7LL;
      dep[b] = (int)(nd > MIX_MAX_DEPTH ? MIX_MAX_DEPTH : nd);
      any = true;
    }
  return any ? mix_set_layout(c, dep, true) : WPIC_OK;
}

double shock_xend(const wpic_ctx* c, double u0);

int mixed_step(wpic_ctx* c) {
  Dev2D& d = c->d;
  if (d.ph.bc == BC_SHOCK) {  // the injection boundary inside the push kernel, in cells from nxgs
    const double xe = shock_xend(c, c->u0) * d.ph.d_delx - (double)d.g.nxgs;
    const double fl = std::floor(xe);
    d.m.k_xend_cell = (int)fl;
    d.m.k_xend_frac = (float)(xe - fl);
    if (d.m.k_xend_frac >= 1.f) {
      d.m.k_xend_frac = 0.f;
      d.m.k_xend_cell += 1;
    }
    d.m.k_u0 = (float)c->u0;
  }
  stage_begin(c, SG_PUSH);
  mix_push_deposit2d(d, c->tmap, c->pusher == WPIC_PUSH_VAY, c->stream);
  stage_end(c, SG_PUSH, 1);
  // the arrivals join their columns right away, so the particle state is whole again before
  // the field solve (which does not read particles) can return an error
  stage_begin(c, SG_PBC);
  mix_migrate2d(d, c->stream);
  stage_end(c, SG_PBC, 1);
  CK(cudaMemcpyAsync(c->h_grow, d.m.grow, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  stage_begin(c, SG_JREDUCE);
  mix_curre_refresh2d(d, c->stream);
  stage_end(c, SG_JREDUCE, d.ph.bc == BC_PERIODIC ? 3 : 2);
  stage_begin(c, SG_FIELD);
  fast::gkl2d(d, c->stream);
  stage_end(c, SG_FIELD, 1);
  int st = do_cg(c);
  if (st) return st;
  stage_begin(c, SG_FIELD);
  dfield_ghost2d(d, c->stream);
  fast::efield2d(d, c->stream);
  dfield_ghost2d(d, c->stream);
  uf_add2d(d, c->stream);
  stage_end(c, SG_FIELD, 6);
  // the CG's host checks synchronised the stream, so the grow flag of this step is in h_grow
  if (*c->h_grow) return mix_grow(c);
  return WPIC_OK;
}

// boundary_shock__injection's right end: xend = nxe dx + v0 dt in the reference's FP64
// expression (2d/proj/shock/boundary_shock.f90:272)
double shock_xend(const wpic_ctx* c, double u0) {
  return shock_xend_value(c->d.g.nxgs + c->d.g.wx1, c->d.ph.delx, u0, c->d.ph.c, c->d.ph.delt);
}

void do_injection(wpic_ctx* c, double u0) {
  stage_begin(c, SG_PBC);
  injection2d(c->d, c->d.B, u0, shock_xend(c, u0), c->stream);
  stage_end(c, SG_PBC, 1);
}

int one_step(wpic_ctx* c) {
  if (c->mixed) return mixed_step(c);
  do_push(c);
  // the shock driver's order (2d/proj/shock/app.f90:110-115): injection before the field
  // solve and no particle_x; the reconnection driver's: particle_x before the field solve
  if (c->d.ph.bc == BC_SHOCK) do_injection(c, c->u0);
  if (c->d.ph.bc == BC_RECONNECTION) do_particle_x(c);
  int st = do_field(c);
  if (st) return st;
  // periodic: particle_x (2d/common/boundary_periodic.f90:61-96) with particle_y's scan
  do_migrate_sort(c, c->d.ph.bc == BC_PERIODIC);
  return WPIC_OK;
}

}  // namespace

namespace {
// The device address of a host array the GPU can read and write in place (page-locked and
// mapped, as wpic_host_register makes it; on Grace the GPU reaches it over NVLink-C2C), or
// null.  The mixed path's conversion kernels then read and write the host rows directly,
// one pass over the link without staging copies.  They move 16 bytes per access, so an array
// that is not 16-byte aligned takes the staged copies instead.
template <typename T>
T* device_view(T* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, (const void*)p) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer || ((size_t)a.devicePointer & 15)) return nullptr;
  return (T*)a.devicePointer;
}
}  // namespace

extern "C" {

int wpic_init_2d(wpic_ctx** out, const wpic_params* p, void* cuda_stream) {
  if (!out || !p) return WPIC_BAD_ARGUMENT;
  *out = nullptr;
  const int nx = p->nxge - p->nxgs + 1, ny = p->nyge - p->nygs + 1;
  if (p->ndim != 6 || p->nsp < 1 || p->nsp > 2 || nx < 4 || ny < 4 || p->np < 1) return WPIC_BAD_ARGUMENT;
  if (p->nys != p->nygs || p->nye != p->nyge) return WPIC_BAD_ARGUMENT;  // one device holds the whole domain
  if (!(p->delx > 0) || !(p->delt > 0) || !(p->c > 0)) return WPIC_BAD_ARGUMENT;
  if (p->bc_kind != WPIC_BC_PERIODIC && p->bc_kind != WPIC_BC_RECONNECTION && p->bc_kind != WPIC_BC_SHOCK)
    return WPIC_BAD_ARGUMENT;
  if (p->precision != WPIC_FP64 && p->precision != WPIC_FP64_EXACT && p->precision != WPIC_MIXED)
    return WPIC_BAD_ARGUMENT;
  if (p->precision == WPIC_MIXED && (nx % MIX_TS != 0 || ny % MIX_TS != 0)) return WPIC_BAD_ARGUMENT;
  wpic_ctx* c = new wpic_ctx();
  c->prm = *p;
  c->mixed = p->precision == WPIC_MIXED;
  Dev2D& d = c->d;
  d.g.nx = nx;
  d.g.ny = ny;
  d.g.nxgs = p->nxgs;
  d.g.nygs = p->nygs;
  d.g.fp = nx + 4;
  d.g.fplane = (nx + 4) * (ny + 4);
  d.g.ncell = nx * ny;
  d.g.wx0 = 0;
  d.g.wx1 = nx - 1;
  Phys& ph = d.ph;
  ph.delx = p->delx;
  ph.delt = p->delt;
  ph.c = p->c;
  ph.gfac = p->gfac;
  ph.nsp = p->nsp;
  ph.bc = p->bc_kind;
  for (int k = 0; k < 2; ++k) {
    ph.q[k] = k < p->nsp ? p->q[k] : 0.0;
    ph.r[k] = k < p->nsp ? p->r[k] : 1.0;
  }
  // field__init constants (2d/common/field.f90:53-59), same operation order
  ph.pi = 4.0 * std::atan(1.0);
  ph.f1 = p->c * p->delt / p->delx;
  ph.f2 = p->gfac * ph.f1 * ph.f1;
  ph.f3 = 4.0 * ph.pi * p->delx / p->c;
  const double t = p->delx / (p->c * p->delt * p->gfac);
  ph.f4 = 4.0 + t * t;
  ph.f5 = t * t;
  ph.d_delx = 1. / p->delx;
  ph.d_delt = 1. / p->delt;
  ph.p_d_delx = 1. / p->delx;
  d.cap = p->device_cap > 0 ? p->device_cap : p->np;
  d.nrowjob = p->nsp * ny;
  d.nred = (d.g.ncell + 255) / 256;
  if (d.nred > 1216) d.nred = 1216;
  d.ite_max = 100;
  d.cg_rtol = 1e-6;  // field.f90:364

  int st = WPIC_OK;
  if (cuda_stream) {
    c->stream = (cudaStream_t)cuda_stream;
  } else {
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete c;
      return WPIC_CUDA_ERROR;
    }
    c->own_stream = true;
  }
  const size_t slots = c->mixed ? 0 : (size_t)d.nrowjob * d.cap;
  const size_t ncell = d.g.ncell, fplane = d.g.fplane;
  d.mixed = c->mixed ? 1 : 0;
  do {
    if (c->mixed) {
      Mix2D& m = d.m;
      m.ntx = nx / MIX_TS;
      m.nty = ny / MIX_TS;
      m.ntile = m.ntx * m.nty;
      m.nbin = m.ntile * p->nsp;
      // largest contribution of one particle to one node of the deposit (sets the fixed-point
      // scales, see mix_set_scales)
      double vmax = 0.0;
      for (int k = 0; k < p->nsp; ++k) {
        const double a = std::fabs(p->q[k]) * p->delx / p->delt, b = 2.0 * std::fabs(p->q[k]) * p->c;
        vmax = std::fmax(vmax, std::fmax(a, b));
      }
      c->mix_vmax = std::fmax(vmax, 1e-300);
      for (int k = 0; k < 2; ++k) {
        const int is = k < p->nsp ? k : 0;
        m.k_fac1[k] = (float)(p->q[is] / p->r[is] * 0.5 * p->delt);
        m.k_fac2[k] = (float)(p->q[is] * p->delt / p->r[is]);
        m.k_qdd[k] = (float)(p->q[is] * p->delx * (1.0 / p->delt));
        m.k_q[k] = (float)p->q[is];
      }
      m.k_dtdx = (float)(p->delt * (1.0 / p->delx));
      m.k_c = (float)p->c;
      m.k_ic2 = (float)(1.0 / (p->c * p->c));
      const size_t ncol = (size_t)m.nbin * MIX_TC;
      if ((st = dalloc(c, &m.boff, m.nbin)) || (st = dalloc(c, &m.bdep, m.nbin)) || (st = dalloc(c, &m.cnt, ncol)) ||
          (st = dalloc(c, &m.ccnt, ncol)) || (st = dalloc(c, &m.acnt, ncol)) || (st = dalloc(c, &m.bneed, m.nbin)) ||
          (st = dalloc(c, &m.grow, 1)) || (st = dalloc(c, &m.ujx, 3 * (size_t)(nx + 4) * (ny + 4))))
        break;
      if (cudaMallocHost(&c->h_grow, sizeof(int)) != cudaSuccess) {
        st = WPIC_CUDA_ERROR;
        break;
      }
      *c->h_grow = 0;
      // an initial layout for the capacity the caller allotted (np per row); put and load
      // lay the bins out again for the particles they bring
      const int dep0 = mix_initial_depth((double)p->np / nx, p->c * p->delt / p->delx);
      if ((st = mix_set_layout(c, std::vector<int>(m.nbin, dep0), false))) break;
    } else {
      if ((st = alloc_parts(c, &d.A, slots))) break;
      if ((st = alloc_parts(c, &d.B, slots))) break;
    }
    if ((st = dalloc(c, &d.cc, (size_t)d.nrowjob * (nx + 1)))) break;
    if ((st = dalloc(c, &d.np2, d.nrowjob))) break;
    if ((st = dalloc(c, &d.np2new, d.nrowjob))) break;
    if ((st = dalloc(c, &d.nup, d.nrowjob))) break;
    if ((st = dalloc(c, &d.ndown, d.nrowjob))) break;
    if ((st = dalloc(c, &d.uf, 6 * fplane))) break;
    if ((st = dalloc(c, &d.df, 6 * fplane))) break;
    if ((st = dalloc(c, &d.uj, 3 * fplane))) break;
    if ((st = dalloc(c, &d.gkl, 3 * ncell))) break;
    if (!c->mixed && (st = dalloc(c, &d.cellJ, 75 * ncell))) break;
    if ((st = dalloc(c, &d.phi, 3 * ncell))) break;
    if ((st = dalloc(c, &d.p, 3 * ncell))) break;
    if ((st = dalloc(c, &d.r, 3 * ncell))) break;
    if ((st = dalloc(c, &d.ap, 3 * ncell))) break;
    if ((st = dalloc(c, &d.b, 3 * ncell))) break;
    if ((st = dalloc(c, &d.partials, (size_t)3 * d.nred * 2))) break;
    if ((st = dalloc(c, &d.cg, 3))) break;
    if ((st = dalloc(c, &d.err, 1))) break;
    if ((st = dalloc(c, &d.red_out, 8))) break;
    if (!c->mixed) {
      if ((st = dalloc(c, &d.mig, slots))) break;
      if ((st = dalloc(c, &d.ulist, slots))) break;
      if ((st = dalloc(c, &d.dlist, slots))) break;
      if ((st = dalloc(c, &d.tlist, slots))) break;
      if ((st = dalloc(c, &d.slist, slots))) break;
      if ((st = dalloc(c, &d.map, slots))) break;
    } else if (mix_setup2d(d, c->tmap) != 0) {
      st = WPIC_CUDA_ERROR;
      break;
    }
    if (cudaMallocHost(&c->h_cg, 3 * sizeof(CGState)) != cudaSuccess) { st = WPIC_CUDA_ERROR; break; }
    if (cudaMallocHost(&c->h_err, sizeof(int)) != cudaSuccess) { st = WPIC_CUDA_ERROR; break; }
    for (int s = 0; s < SG_COUNT; ++s) {
      cudaEventCreate(&c->ev0[s]);
      cudaEventCreate(&c->ev1[s]);
    }
  } while (0);
  if (st == WPIC_OK) st = cuda_status(cudaStreamSynchronize(c->stream));
  if (st != WPIC_OK) {
    wpic_finalize(c);
    return st;
  }
  *out = c;
  return WPIC_OK;
}

int wpic_finalize(wpic_ctx* c) {
  if (!c) return WPIC_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (void* p : c->allocs) cudaFree(p);
  if (c->mixP) cudaFree(c->mixP);
  if (c->adj_fields) cudaFree(c->adj_fields);
  if (c->h_grow) cudaFreeHost(c->h_grow);
  for (int k = 0; k < 2; ++k)
    if (c->xfer[k]) cudaStreamSynchronize(c->xfer[k]);
  for (int k = 0; k < 2; ++k) {
    if (c->xstg[k]) cudaFree(c->xstg[k]);
    for (int q = 0; q < 2; ++q)
      if (c->ev_copied[k][q]) cudaEventDestroy(c->ev_copied[k][q]);
    if (c->ev_used[k]) cudaEventDestroy(c->ev_used[k]);
    if (c->xfer[k]) cudaStreamDestroy(c->xfer[k]);
  }
  if (c->staging) cudaFree(c->staging);
  if (c->h_cg) cudaFreeHost(c->h_cg);
  if (c->h_err) cudaFreeHost(c->h_err);
  for (int s = 0; s < SG_COUNT; ++s) {
    if (c->ev0[s]) cudaEventDestroy(c->ev0[s]);
    if (c->ev1[s]) cudaEventDestroy(c->ev1[s]);
  }
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return WPIC_OK;
}

int wpic_put_particles(wpic_ctx* c, int which, const double* up, const int* np2, const int* cumcnt) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (!up || !np2 || (which == 0 && !cumcnt) || (which != 0 && which != 1)) return WPIC_BAD_ARGUMENT;
  Dev2D& d = c->d;
  const int nx = d.g.nx, ndim = c->prm.ndim, nph = c->prm.np;
  for (int r = 0; r < d.nrowjob; ++r)
    if (np2[r] < 0 || np2[r] > d.cap || np2[r] > nph) return WPIC_CAPACITY;
  // cumcnt: prefix sums of the rows' cell counts (checked while the first copies run in the mixed path)
  auto check_cumcnt = [&]() -> int {
    if (which != 0) return WPIC_OK;
    for (int r = 0; r < d.nrowjob; ++r) {
      const int* cc = cumcnt + (size_t)r * (nx + 1);
      if (cc[0] != 0 || cc[nx] != np2[r]) return WPIC_BAD_ARGUMENT;
      for (int i = 0; i < nx; ++i)
        if (cc[i + 1] < cc[i]) return WPIC_BAD_ARGUMENT;
    }
    return WPIC_OK;
  };
  if (c->mixed && which == 1) {
    // the unsorted state of the restart path (io__input's up, before sort__bucket; the rows
    // are right, the order within a row is not): each row is bucket-sorted on the host by
    // its x cell i = int(x) as sort__bucket does (2d/common/sort.f90:60), stably, and put as
    // the sorted state, which is all a mixed context keeps
    std::vector<double> sorted((size_t)d.nrowjob * ndim * nph);
    std::vector<int> cc((size_t)d.nrowjob * (nx + 1));
    std::vector<int> cell(nph);
    for (int r = 0; r < d.nrowjob; ++r) {
      const double* row = up + (size_t)r * ndim * nph;
      int* crow = cc.data() + (size_t)r * (nx + 1);
      std::fill(crow, crow + nx + 1, 0);
      for (int k = 0; k < np2[r]; ++k) {
        const double x = row[(size_t)k * ndim];
        int i = (x > -2147483648.0 && x < 2147483647.0) ? (int)x - d.g.nxgs : -1;
        if (i < 0 || i >= nx) return WPIC_OUT_OF_RANGE;
        cell[k] = i;
        ++crow[i + 1];
      }
      for (int i = 0; i < nx; ++i) crow[i + 1] += crow[i];
      std::vector<int> next(crow, crow + nx);
      double* out = sorted.data() + (size_t)r * ndim * nph;
      for (int k = 0; k < np2[r]; ++k)
        std::copy(row + (size_t)k * ndim, row + (size_t)(k + 1) * ndim, out + (size_t)(next[cell[k]]++) * ndim);
    }
    return wpic_put_particles(c, 0, sorted.data(), np2, cc.data());
  }
  if (!c->mixed) {
    const int st = check_cumcnt();
    if (st) return st;
  }
  CK(cudaMemcpyAsync(d.np2, np2, sizeof(int) * d.nrowjob, cudaMemcpyHostToDevice, c->stream));
  if (which == 0)
    CK(cudaMemcpyAsync(d.cc, cumcnt, sizeof(int) * (size_t)d.nrowjob * (nx + 1), cudaMemcpyHostToDevice,
                       c->stream));
  const size_t row_bytes = (size_t)ndim * nph * sizeof(double);
  if (c->mixed) {
    int st = ensure_xfer(c, (size_t)MIX_TS * row_bytes);
    if (st) return st;
    // the first two chunks start crossing the link while the device finds each bin's fullest
    // cell (the layout check below); their staging buffers are free (the last call finished)
    auto copy_chunk = [&](int k) -> int {
      const int isp = k / d.m.nty, ty = k - isp * d.m.nty;
      const size_t r0 = (size_t)isp * d.g.ny + (size_t)ty * MIX_TS;
      for (int rr = 0; rr < MIX_TS; ++rr) {
        const size_t nb = (size_t)np2[r0 + rr] * ndim * sizeof(double);
        if (nb)
          CK(cudaMemcpyAsync(c->xstg[k & 1] + (size_t)rr * nph * ndim, up + (r0 + rr) * ndim * nph, nb,
                             cudaMemcpyHostToDevice, c->xfer[rr & 1]));
      }
      for (int q = 0; q < 2; ++q) CK(cudaEventRecord(c->ev_copied[k & 1][q], c->xfer[q]));
      return WPIC_OK;
    };
    const int nchunk = c->prm.nsp * d.m.nty;
    const double* dv = device_view(up);
    for (int k = 0; k < 2 && k < nchunk && !dv; ++k)
      if ((st = copy_chunk(k))) return st;
    if ((st = check_cumcnt())) {
      sync_xfer(c);
      return st;
    }
    // lay the bins out for these particles unless every bin already has the room: each bin's
    // depth from its fullest cell
    {
      const Mix2D& m = d.m;
      mix_binmax2d(d, c->stream);
      std::vector<int> mx(m.nbin);
      CK(cudaMemcpyAsync(mx.data(), m.bneed, sizeof(int) * m.nbin, cudaMemcpyDeviceToHost, c->stream));
      CK(cudaStreamSynchronize(c->stream));
      const double cdx = c->prm.c * c->prm.delt / c->prm.delx;
      // the current layout is kept while every bin keeps 40 % of its depth free above its
      // fullest cell (room for the arrivals of the next steps; bins grow on demand after that)
      std::vector<int> dep(m.nbin);
      bool fits = (int)c->h_dep.size() == m.nbin;
      for (int b = 0; b < m.nbin; ++b) {
        dep[b] = mix_initial_depth(mx[b], cdx);
        if (fits && 5LL * mx[b] > 3LL * c->h_dep[b]) fits = false;
      }
      if (!fits && (st = mix_set_layout(c, dep, false))) return st;
    }
    if (dv) {  // the conversion kernels read the host rows in place
      for (int isp = 0; isp < c->prm.nsp; ++isp)
        mix_put2d(d, dv + (size_t)isp * d.g.ny * ndim * nph, ndim, nph, isp, 0, d.m.nty, c->stream);
      return finish(c);
    }
    // one tile row (16 bucket rows) of one species per chunk: the valid prefix of each row is
    // copied into staging buffer k % 2 on the copy stream while the device converts chunk k - 1
    for (int k = 0; k < nchunk; ++k) {
      const int b = k & 1;
      const int isp = k / d.m.nty, ty = k - isp * d.m.nty;
      if (k >= 2) {
        for (int q = 0; q < 2; ++q) CK(cudaStreamWaitEvent(c->xfer[q], c->ev_used[b], 0));
        if ((st = copy_chunk(k))) return st;
      }
      for (int q = 0; q < 2; ++q) CK(cudaStreamWaitEvent(c->stream, c->ev_copied[b][q], 0));
      mix_put2d(d, c->xstg[b], ndim, nph, isp, ty, 1, c->stream);
      CK(cudaEventRecord(c->ev_used[b], c->stream));
    }
    if ((st = sync_xfer(c))) return st;
    return finish(c);
  }
  size_t rows_per = ((size_t)1 << 30) / row_bytes;
  if (rows_per < 1) rows_per = 1;
  if (rows_per > (size_t)d.nrowjob) rows_per = d.nrowjob;
  int st = ensure_staging(c, rows_per * row_bytes);
  if (st) return st;
  const Parts64& P = which == 0 ? d.A : d.B;
  for (int r0 = 0; r0 < d.nrowjob; r0 += (int)rows_per) {
    const int nr = (int)((size_t)(d.nrowjob - r0) < rows_per ? d.nrowjob - r0 : rows_per);
    CK(cudaMemcpyAsync(c->staging, up + (size_t)r0 * ndim * nph, nr * row_bytes, cudaMemcpyHostToDevice,
                       c->stream));
    aos_to_soa2d(d, c->staging, ndim, nph, r0, nr, P, c->stream);
  }
  return finish(c);
}

int wpic_get_particles(wpic_ctx* c, int which, double* up, int* np2, int* cumcnt) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (!up || (which != 0 && which != 1)) return WPIC_BAD_ARGUMENT;
  Dev2D& d = c->d;
  const int nx = d.g.nx, ndim = c->prm.ndim, nph = c->prm.np;
  if (c->mixed) {
    if (which != 0) return WPIC_BAD_ARGUMENT;
    mix_count_rows2d(d, c->stream);
    c->h_np2.resize(d.nrowjob);
    CK(cudaMemcpyAsync(c->h_np2.data(), d.np2, sizeof(int) * d.nrowjob, cudaMemcpyDeviceToHost, c->stream));
    if (cumcnt)
      CK(cudaMemcpyAsync(cumcnt, d.cc, sizeof(int) * (size_t)d.nrowjob * (nx + 1), cudaMemcpyDeviceToHost,
                         c->stream));
    CK(cudaStreamSynchronize(c->stream));  // the row counts size the copies below
    for (int r = 0; r < d.nrowjob; ++r)
      if (c->h_np2[r] > nph) return WPIC_CAPACITY;
    if (np2) std::copy(c->h_np2.begin(), c->h_np2.end(), np2);
    if (double* dv = device_view(up)) {  // the kernels write the host rows in place
      for (int isp = 0; isp < c->prm.nsp; ++isp)
        mix_get2d(d, dv + (size_t)isp * d.g.ny * ndim * nph, ndim, nph, isp, 0, d.m.nty, c->stream);
      return finish(c);
    }
    const size_t row_bytes = (size_t)ndim * nph * sizeof(double);
    // chunk k is converted into staging buffer k % 2 while the copy stream moves chunk k - 1
    // to the host; only each row's valid prefix crosses the link
    int st = ensure_xfer(c, (size_t)MIX_TS * row_bytes);
    if (st) return st;
    int k = 0;
    for (int isp = 0; isp < c->prm.nsp; ++isp)
      for (int ty = 0; ty < d.m.nty; ++ty, ++k) {
        const int b = k & 1;
        const size_t r0 = (size_t)isp * d.g.ny + (size_t)ty * MIX_TS;
        if (k >= 2)
          for (int q = 0; q < 2; ++q) CK(cudaStreamWaitEvent(c->stream, c->ev_copied[b][q], 0));
        mix_get2d(d, c->xstg[b], ndim, nph, isp, ty, 1, c->stream);
        CK(cudaEventRecord(c->ev_used[b], c->stream));
        for (int q = 0; q < 2; ++q) CK(cudaStreamWaitEvent(c->xfer[q], c->ev_used[b], 0));
        for (int rr = 0; rr < MIX_TS; ++rr) {
          const size_t nb = (size_t)c->h_np2[r0 + rr] * ndim * sizeof(double);
          if (nb)
            CK(cudaMemcpyAsync(up + (r0 + rr) * ndim * nph, c->xstg[b] + (size_t)rr * nph * ndim, nb,
                               cudaMemcpyDeviceToHost, c->xfer[rr & 1]));
        }
        for (int q = 0; q < 2; ++q) CK(cudaEventRecord(c->ev_copied[b][q], c->xfer[q]));
      }
    if ((st = sync_xfer(c))) return st;
    return finish(c);
  }
  if (np2) CK(cudaMemcpyAsync(np2, d.np2, sizeof(int) * d.nrowjob, cudaMemcpyDeviceToHost, c->stream));
  if (cumcnt && which == 0)
    CK(cudaMemcpyAsync(cumcnt, d.cc, sizeof(int) * (size_t)d.nrowjob * (nx + 1), cudaMemcpyDeviceToHost,
                       c->stream));
  const size_t row_bytes = (size_t)ndim * nph * sizeof(double);
  size_t rows_per = ((size_t)1 << 30) / row_bytes;
  if (rows_per < 1) rows_per = 1;
  if (rows_per > (size_t)d.nrowjob) rows_per = d.nrowjob;
  int st = ensure_staging(c, rows_per * row_bytes);
  if (st) return st;
  const Parts64& P = which == 0 ? d.A : d.B;
  for (int r0 = 0; r0 < d.nrowjob; r0 += (int)rows_per) {
    const int nr = (int)((size_t)(d.nrowjob - r0) < rows_per ? d.nrowjob - r0 : rows_per);
    soa_to_aos2d(d, c->staging, ndim, nph, r0, nr, P, c->stream);
    CK(cudaMemcpyAsync(up + (size_t)r0 * ndim * nph, c->staging, nr * row_bytes, cudaMemcpyDeviceToHost,
                       c->stream));
  }
  return finish(c);
}

static int put_field(wpic_ctx* c, const double* ref, double* dst, int ncomp) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (!ref) return WPIC_BAD_ARGUMENT;
  const size_t n = (size_t)ncomp * c->d.g.fplane;
  int st = ensure_staging(c, n * sizeof(double));
  if (st) return st;
  CK(cudaMemcpyAsync(c->staging, ref, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  field_ref_to_soa(c->staging, dst, ncomp, c->d.g.fplane, c->stream);
  return finish(c);
}

static int get_field(wpic_ctx* c, double* ref, const double* src, int ncomp) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (!ref) return WPIC_BAD_ARGUMENT;
  const size_t n = (size_t)ncomp * c->d.g.fplane;
  int st = ensure_staging(c, n * sizeof(double));
  if (st) return st;
  field_soa_to_ref(src, c->staging, ncomp, c->d.g.fplane, c->stream);
  CK(cudaMemcpyAsync(ref, c->staging, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  return finish(c);
}

// ---------------------------------------------------------------------------
// adjoint of nsteps fused steps (FP64, periodic): states every `every` steps are kept; each
// segment is recomputed forward with every step's state stored, then swept backwards with
// the kernels of adjoint2d.cu.  The gradients are of the scalar whose gradient with respect
// to the final fields is lam_uf_final (reference layout); they are returned with respect to
// the particle state (same layout as wpic_get_particles: x, y, ux, uy, uz; the id column
// carries the ids) and the fields at the start.  The context ends in its final state.
// ---------------------------------------------------------------------------
namespace {

int adj_alloc_state(wpic_ctx* c, wpic_ctx::AdjState& S) {
  const Dev2D& d = c->d;
  const size_t slots = (size_t)d.nrowjob * d.cap;
  int st;
  if ((st = alloc_parts(c, &S.A, slots))) return st;
  if ((st = dalloc(c, &S.cc, (size_t)d.nrowjob * (d.g.nx + 1)))) return st;
  if ((st = dalloc(c, &S.np2, (size_t)d.nrowjob))) return st;
  if ((st = dalloc(c, &S.uf, 6 * (size_t)d.g.fplane))) return st;
  return dalloc(c, &S.df, 6 * (size_t)d.g.fplane);
}

void adj_copy_parts(const Parts64& from, const Parts64& to, size_t n, cudaStream_t s) {
  cudaMemcpyAsync(to.x, from.x, n * 8, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(to.y, from.y, n * 8, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(to.ux, from.ux, n * 8, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(to.uy, from.uy, n * 8, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(to.uz, from.uz, n * 8, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(to.id, from.id, n * 8, cudaMemcpyDeviceToDevice, s);
}

void adj_save(wpic_ctx* c, const wpic_ctx::AdjState& S) {
  Dev2D& d = c->d;
  const size_t slots = (size_t)d.nrowjob * d.cap;
  adj_copy_parts(d.A, S.A, slots, c->stream);
  cudaMemcpyAsync(S.cc, d.cc, sizeof(int) * (size_t)d.nrowjob * (d.g.nx + 1), cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(S.np2, d.np2, sizeof(int) * (size_t)d.nrowjob, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(S.uf, d.uf, sizeof(double) * 6 * (size_t)d.g.fplane, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(S.df, d.df, sizeof(double) * 6 * (size_t)d.g.fplane, cudaMemcpyDeviceToDevice, c->stream);
}

// the pushed particles and the permutation of one step, kept for its adjoint
int adj_alloc_step(wpic_ctx* c, wpic_ctx::AdjState& S) {
  if (S.map) return WPIC_OK;
  const Dev2D& d = c->d;
  const size_t slots = (size_t)d.nrowjob * d.cap;
  int st;
  if ((st = dalloc(c, &S.B.x, slots)) || (st = dalloc(c, &S.B.y, slots)) || (st = dalloc(c, &S.B.ux, slots)) ||
      (st = dalloc(c, &S.B.uy, slots)) || (st = dalloc(c, &S.B.uz, slots)) || (st = dalloc(c, &S.np2new, d.nrowjob)))
    return st;
  return dalloc(c, &S.map, slots);
}

// The field store for n states (12 field planes each), when it fits in half of the free device
// memory; otherwise no store (adj_nfield 0) and the segments are recomputed in full.
int adj_field_store(wpic_ctx* c, int n) {
  c->adj_nfield = 0;
  if (n < 1 || !c->adj_keep_fields) return WPIC_OK;
  const size_t per = 12 * (size_t)c->d.g.fplane;
  if ((size_t)n > c->adj_fields_slots) {
    CK(cudaStreamSynchronize(c->stream));
    if (c->adj_fields) cudaFree(c->adj_fields);
    c->adj_fields = nullptr;
    c->adj_fields_slots = 0;
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    if ((size_t)n * per * sizeof(double) > free_b / 2) return WPIC_OK;
    void* v = nullptr;
    if (cudaMalloc(&v, (size_t)n * per * sizeof(double)) != cudaSuccess) {
      (void)cudaGetLastError();  // no store: the recompute runs the full step
      return WPIC_OK;
    }
    c->adj_fields = (double*)v;
    c->adj_fields_slots = n;
  }
  c->adj_nfield = n;
  return WPIC_OK;
}

// the field state before step j (1 <= j <= adj_nfield) of the recorded run: into slot j - 1, or back
void adj_field_slot(wpic_ctx* c, int j, bool save) {
  Dev2D& d = c->d;
  const size_t P6 = 6 * (size_t)d.g.fplane;
  double* const f = c->adj_fields + (size_t)(j - 1) * 2 * P6;
  const cudaMemcpyKind k = cudaMemcpyDeviceToDevice;
  cudaMemcpyAsync(save ? f : d.uf, save ? d.uf : f, P6 * sizeof(double), k, c->stream);
  cudaMemcpyAsync(save ? f + P6 : d.df, save ? d.df : f + P6, P6 * sizeof(double), k, c->stream);
}

// one periodic step (one_step's order) that keeps B after the push and the sort's permutation;
// replay > 0: the fields after the step are the stored state `replay` of the recorded run (the
// same values the deposit and the solve gave then), so neither runs
int adj_forward_step(wpic_ctx* c, wpic_ctx::AdjState& S, int replay = 0) {
  Dev2D& d = c->d;
  const size_t slots = (size_t)d.nrowjob * d.cap;
  do_push(c);
  for (int q = 0; q < 5; ++q) {
    double* const from[5] = {d.B.x, d.B.y, d.B.ux, d.B.uy, d.B.uz};
    double* const to[5] = {S.B.x, S.B.y, S.B.ux, S.B.uy, S.B.uz};
    cudaMemcpyAsync(to[q], from[q], slots * 8, cudaMemcpyDeviceToDevice, c->stream);
  }
  if (replay > 0) {
    adj_field_slot(c, replay, false);
  } else {
    int st = do_field(c);
    if (st) return st;
  }
  do_migrate_sort(c, true);  // periodic: particle_x with particle_y's scan
  cudaMemcpyAsync(S.map, d.map, slots * sizeof(int), cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(S.np2new, d.np2new, (size_t)d.nrowjob * sizeof(int), cudaMemcpyDeviceToDevice, c->stream);
  S.has_step = true;
  return WPIC_OK;
}

void adj_load(wpic_ctx* c, const wpic_ctx::AdjState& S) {
  Dev2D& d = c->d;
  const size_t slots = (size_t)d.nrowjob * d.cap;
  adj_copy_parts(S.A, d.A, slots, c->stream);
  cudaMemcpyAsync(d.cc, S.cc, sizeof(int) * (size_t)d.nrowjob * (d.g.nx + 1), cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(d.np2, S.np2, sizeof(int) * (size_t)d.nrowjob, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(d.uf, S.uf, sizeof(double) * 6 * (size_t)d.g.fplane, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(d.df, S.df, sizeof(double) * 6 * (size_t)d.g.fplane, cudaMemcpyDeviceToDevice, c->stream);
}

int adj_prepare(wpic_ctx* c, int nstates) {
  Dev2D& d = c->d;
  int st;
  if (!c->adj_ready) {
    const size_t slots = (size_t)d.nrowjob * d.cap, P = d.g.fplane;
    const size_t nt = 6 * (size_t)(d.g.nx + 2) * (d.g.ny + 2);
    if ((st = alloc_parts(c, &c->lA, slots)) || (st = alloc_parts(c, &c->lB, slots))) return st;
    if ((st = dalloc(c, &c->luf, 6 * P)) || (st = dalloc(c, &c->ldf, 6 * P)) || (st = dalloc(c, &c->luj, 3 * P)))
      return st;
    if ((st = dalloc(c, &c->lg, 3 * (size_t)d.g.ncell)) || (st = dalloc(c, &c->tmpc, nt)) ||
        (st = dalloc(c, &c->ltmp, nt)) || (st = dalloc(c, &c->adj_cc, (size_t)d.nrowjob * (d.g.nx + 1))) ||
        (st = dalloc(c, &c->adj_f32, 6 * P)))
      return st;
    if ((st = ensure_C(c))) return st;
    c->adj_ready = true;
  }
  while ((int)c->adj_states.size() < nstates) {
    wpic_ctx::AdjState S{};
    if ((st = adj_alloc_state(c, S))) return st;
    c->adj_states.push_back(S);
  }
  return WPIC_OK;
}

// the self-checks' scratch: 8 dot-product slots, four particle sets, two field and one current array
int chk_scratch(wpic_ctx* c, bool parts, bool fields) {
  const Dev2D& d = c->d;
  const size_t P = d.g.fplane, slots = (size_t)d.nrowjob * d.cap;
  int st;
  if (!c->chk_dots && (st = dalloc(c, &c->chk_dots, 8))) return st;
  if (parts && !c->chk_A0.x &&
      ((st = alloc_parts(c, &c->chk_A0, slots)) || (st = alloc_parts(c, &c->chk_B0, slots)) ||
       (st = alloc_parts(c, &c->chk_vA, slots)) || (st = alloc_parts(c, &c->chk_vB, slots))))
    return st;
  if (fields && !c->chk_f0 &&
      ((st = dalloc(c, &c->chk_f0, 6 * P)) || (st = dalloc(c, &c->chk_v, 6 * P)) || (st = dalloc(c, &c->chk_lj, 3 * P))))
    return st;
  return WPIC_OK;
}

void adj_zero_parts(const Parts64& P, size_t n, cudaStream_t s) {
  cudaMemsetAsync(P.x, 0, n * 8, s);
  cudaMemsetAsync(P.y, 0, n * 8, s);
  cudaMemsetAsync(P.ux, 0, n * 8, s);
  cudaMemsetAsync(P.uy, 0, n * 8, s);
  cudaMemsetAsync(P.uz, 0, n * 8, s);
}

// one step backwards: d holds the state before the step; lA, luf hold the adjoints of the
// state after it and return those of the state before it
int adj_step(wpic_ctx* c, const wpic_ctx::AdjState* S) {
  Dev2D& d = c->d;
  const size_t slots = (size_t)d.nrowjob * d.cap;
  if (S && S->has_step) {
    // B and the permutation kept by the recompute: the adjoint runs on them in place
    const Parts64 B0 = d.B;
    int* const map0 = d.map;
    int* const np2new0 = d.np2new;
    d.B = S->B;
    d.B.id = B0.id;
    d.map = S->map;
    d.np2new = S->np2new;
    // the unsort writes every valid slot of lB (the step's permutation is a bijection)
    adj_unsort(d, c->lA, c->lB, c->stream);
    adj_zero_parts(c->lA, slots, c->stream);
    adj_field(d, c->luf, c->ldf, c->luj, c->stream);
    int st = do_cg(c);
    if (!st) {
      adj_field_after_cg(d, c->luf, c->lg, c->luj, c->stream);
      adj_particles(d, c->luj, c->lA, c->lB, c->tmpc, c->ltmp, c->luf, c->adj_fp32 ? c->adj_f32 : nullptr, c->stream);
    }
    d.B = B0;
    d.map = map0;
    d.np2new = np2new0;
    return st;
  }
  fast::push2d(d, c->stream);                        // B: the pushed particles, before the wraps
  adj_copy_parts(d.B, d.C, slots, c->stream);        // the bookkeeping on a copy gives the permutation
  const size_t ccb = (size_t)d.nrowjob * (d.g.nx + 1) * sizeof(int);
  cudaMemcpyAsync(c->adj_cc, d.cc, ccb, cudaMemcpyDeviceToDevice, c->stream);  // the sort rewrites cc
  wrapx_migrate_scan2d(d, d.C, c->stream);
  migrate_plan2d(d, c->stream);
  sort_rank2d(d, d.C, d.slist, c->stream);
  adj_unsort(d, c->lA, c->lB, c->stream);  // writes every valid slot of lB
  cudaMemcpyAsync(d.cc, c->adj_cc, ccb, cudaMemcpyDeviceToDevice, c->stream);  // the deposit and push read it
  adj_zero_parts(c->lA, slots, c->stream);
  adj_field(d, c->luf, c->ldf, c->luj, c->stream);
  int st = do_cg(c);                                 // the adjoint solve: same symmetric operator
  if (st) return st;
  adj_field_after_cg(d, c->luf, c->lg, c->luj, c->stream);
  adj_particles(d, c->luj, c->lA, c->lB, c->tmpc, c->ltmp, c->luf, c->adj_fp32 ? c->adj_f32 : nullptr, c->stream);
  return WPIC_OK;
}

}  // namespace

// <L x, y> against <x, L^T y> for the transposed linear operators of the field part, with
// random vectors: out[0] current fold, out[1] ghost copies, out[2] E update, out[3] RHS,
// out[4] tmp averaging (relative differences).  Overwrites the context's fields.
int wpic_adjoint_selfcheck(wpic_ctx* c, double* out) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mixed || c->d.ph.bc != BC_PERIODIC || !out) return WPIC_BAD_ARGUMENT;
  Dev2D& d = c->d;
  int st = adj_prepare(c, 0);
  if (st) return st;
  const size_t P = d.g.fplane, nc = d.g.ncell, nt = 6 * (size_t)(d.g.nx + 2) * (d.g.ny + 2);
  if ((st = chk_scratch(c, false, false))) return st;
  double* const dots = c->chk_dots;
  double h[8];
  auto dot = [&](const double* a, const double* b, size_t n, int slot) { adj_dot(a, b, n, dots + slot, c->stream); };
  // x in the scratch of the adjoint (luf/ldf/luj/lg: the inputs), y random, forward on d's buffers
  // 0: fold.  x = uj (3P), L x = fold(uj); y = luj
  cudaMemsetAsync(dots, 0, 8 * sizeof(double), c->stream);
  adj_fill_rand(d.uj, 3 * P, 11, c->stream);
  cudaMemcpyAsync(c->ldf, d.uj, 3 * P * 8, cudaMemcpyDeviceToDevice, c->stream);  // keep x
  curre_fold2d(d, c->stream);
  adj_fill_rand(c->luj, 3 * P, 12, c->stream);
  dot(d.uj, c->luj, 3 * P, 0);
  adj_field_fold_T(d, c->luj, c->stream);
  dot(c->ldf, c->luj, 3 * P, 1);
  // 1: ghost copies on 6 components.  x = df, L x = ghost(df); y = ldf
  adj_fill_rand(d.df, 6 * P, 13, c->stream);
  cudaMemcpyAsync(c->luf, d.df, 6 * P * 8, cudaMemcpyDeviceToDevice, c->stream);
  dfield_ghost2d(d, c->stream);
  adj_fill_rand(c->ldf, 6 * P, 14, c->stream);
  dot(d.df, c->ldf, 6 * P, 2);
  adj_field_ghost_T(d, c->ldf, c->stream);
  dot(c->luf, c->ldf, 6 * P, 3);
  CK(cudaMemcpyAsync(h, dots, 4 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  out[0] = std::fabs(h[0] - h[1]) / std::fmax(std::fabs(h[0]), 1e-300);
  out[1] = std::fabs(h[2] - h[3]) / std::fmax(std::fabs(h[2]), 1e-300);
  // 2: E update.  x = (df0..2, uf, uj) random; L x = df3..5 interior; y on df3..5 interior
  cudaMemsetAsync(dots, 0, 8 * sizeof(double), c->stream);
  adj_fill_rand(d.df, 6 * P, 15, c->stream);
  adj_fill_rand(d.uf, 6 * P, 16, c->stream);
  adj_fill_rand(d.uj, 3 * P, 17, c->stream);
  cudaMemsetAsync(d.df + 3 * P, 0, 3 * P * 8, c->stream);
  fast::efield2d(d, c->stream);
  adj_fill_rand(c->ldf, 6 * P, 18, c->stream);
  adj_keep_interior(d, c->ldf + 3 * P, 3, c->stream);  // y: interior of df3..5 only
  cudaMemsetAsync(c->ldf, 0, 3 * P * 8, c->stream);
  dot(d.df + 3 * P, c->ldf + 3 * P, 3 * P, 0);
  cudaMemsetAsync(c->luf, 0, 6 * P * 8, c->stream);
  cudaMemsetAsync(c->luj, 0, 3 * P * 8, c->stream);
  adj_field_efield_T(d, c->ldf, c->luf, c->luj, c->stream);
  dot(d.df, c->ldf, 3 * P, 1);
  dot(d.uf, c->luf, 6 * P, 1);
  dot(d.uj, c->luj, 3 * P, 1);
  // 3: RHS.  x = (uf, uj); L x = gkl; y = lg
  adj_fill_rand(d.uf, 6 * P, 19, c->stream);
  adj_fill_rand(d.uj, 3 * P, 20, c->stream);
  fast::gkl2d(d, c->stream);
  adj_fill_rand(c->lg, 3 * nc, 21, c->stream);
  dot(d.gkl, c->lg, 3 * nc, 2);
  cudaMemsetAsync(c->luf, 0, 6 * P * 8, c->stream);
  cudaMemsetAsync(c->luj, 0, 3 * P * 8, c->stream);
  adj_field_gkl_T(d, c->lg, c->luf, c->luj, c->stream);
  dot(d.uf, c->luf, 6 * P, 3);
  dot(d.uj, c->luj, 3 * P, 3);
  // 4: tmp averaging.  x = uf; L x = tmp; y = ltmp
  adj_fill_rand(d.uf, 6 * P, 22, c->stream);
  adj_field_tmp(d, c->tmpc, c->stream);
  adj_fill_rand(c->ltmp, nt, 23, c->stream);
  dot(c->tmpc, c->ltmp, nt, 4);
  cudaMemsetAsync(c->luf, 0, 6 * P * 8, c->stream);
  adj_field_tmp_T(d, c->ltmp, c->luf, c->stream);
  dot(d.uf, c->luf, 6 * P, 5);
  CK(cudaMemcpyAsync(h, dots, 6 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  out[2] = std::fabs(h[0] - h[1]) / std::fmax(std::fabs(h[0]), 1e-300);
  out[3] = std::fabs(h[2] - h[3]) / std::fmax(std::fabs(h[2]), 1e-300);
  out[4] = std::fabs(h[4] - h[5]) / std::fmax(std::fabs(h[4]), 1e-300);
  return finish(c);
}

// central difference of the push along a random field direction v, projected on a random lB,
// against <v, (dB/duf)^T lB> from the adjoint kernels: out[0] the difference, out[1] the
// adjoint.  Uses the context's particles and fields; the fields are restored.
int wpic_adjoint_pushcheck(wpic_ctx* c, double hstep, double* out) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mixed || !out || !(hstep > 0)) return WPIC_BAD_ARGUMENT;
  Dev2D& d = c->d;
  int st = adj_prepare(c, 0);
  if (st) return st;
  const size_t P = d.g.fplane, slots = (size_t)d.nrowjob * d.cap;
  if ((st = chk_scratch(c, false, false))) return st;
  double* const dots = c->chk_dots;
  cudaMemsetAsync(dots, 0, 4 * sizeof(double), c->stream);
  cudaMemcpyAsync(c->ldf, d.uf, 6 * P * 8, cudaMemcpyDeviceToDevice, c->stream);  // u
  adj_fill_rand(c->luj, 3 * P, 31, c->stream);                                     // v (B components)
  cudaMemsetAsync(c->luf, 0, 6 * P * 8, c->stream);
  cudaMemcpyAsync(c->luf, c->luj, 3 * P * 8, cudaMemcpyDeviceToDevice, c->stream);
  adj_fill_rand(c->luj, 3 * P, 37, c->stream);                                     // v (E components)
  cudaMemcpyAsync(c->luf + 3 * P, c->luj, 3 * P * 8, cudaMemcpyDeviceToDevice, c->stream);
  adj_fill_rand(c->lB.x, slots, 32, c->stream);
  adj_fill_rand(c->lB.y, slots, 33, c->stream);
  adj_fill_rand(c->lB.ux, slots, 34, c->stream);
  adj_fill_rand(c->lB.uy, slots, 35, c->stream);
  adj_fill_rand(c->lB.uz, slots, 36, c->stream);
  adj_axpy(d.uf, c->ldf, c->luf, hstep, 6 * P, c->stream);
  fast::push2d(d, c->stream);
  adj_dot_parts(d, c->lB, d.B, 0.5 / hstep, dots, c->stream);
  adj_axpy(d.uf, c->ldf, c->luf, -hstep, 6 * P, c->stream);
  fast::push2d(d, c->stream);
  adj_dot_parts(d, c->lB, d.B, -0.5 / hstep, dots, c->stream);
  cudaMemcpyAsync(d.uf, c->ldf, 6 * P * 8, cudaMemcpyDeviceToDevice, c->stream);
  // adjoint into ldf (zeroed): <v, ldf>
  cudaMemsetAsync(c->ldf, 0, 6 * P * 8, c->stream);
  adj_push_fields(d, c->lB, c->lA, c->tmpc, c->ltmp, c->ldf, c->adj_fp32 ? c->adj_f32 : nullptr, c->stream);
  adj_dot(c->luf, c->ldf, 6 * P, dots + 1, c->stream);
  double h[2];
  CK(cudaMemcpyAsync(h, dots, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  out[0] = h[0];
  out[1] = h[1];
  return finish(c);
}

// central difference of <lJ, J(A, B)> (J the raw deposit, B the push of the context's state)
// along random directions of A's positions and B's positions and momenta, against the
// deposit's adjoint: out2 = {difference, adjoint}.  The particles are restored.
int wpic_adjoint_depositcheck(wpic_ctx* c, double hstep, double* out) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mixed || !out || !(hstep > 0)) return WPIC_BAD_ARGUMENT;
  Dev2D& d = c->d;
  int st = adj_prepare(c, 0);
  if (st) return st;
  const size_t P = d.g.fplane, slots = (size_t)d.nrowjob * d.cap;
  if ((st = chk_scratch(c, true, false))) return st;
  const Parts64 A0 = c->chk_A0, B0 = c->chk_B0, vA = c->chk_vA, vB = c->chk_vB;
  double* const dots = c->chk_dots;
  cudaMemsetAsync(dots, 0, 4 * sizeof(double), c->stream);
  fast::push2d(d, c->stream);
  adj_copy_parts(d.A, A0, slots, c->stream);
  adj_copy_parts(d.B, B0, slots, c->stream);
  double* va[2] = {vA.x, vA.y};
  double* vb[5] = {vB.x, vB.y, vB.ux, vB.uy, vB.uz};
  double* a_[2] = {d.A.x, d.A.y};
  double* a0[2] = {A0.x, A0.y};
  double* b_[5] = {d.B.x, d.B.y, d.B.ux, d.B.uy, d.B.uz};
  double* b0[5] = {B0.x, B0.y, B0.ux, B0.uy, B0.uz};
  for (int q = 0; q < 2; ++q) adj_fill_rand(va[q], slots, 41 + q, c->stream);
  for (int q = 0; q < 5; ++q) adj_fill_rand(vb[q], slots, 43 + q, c->stream);
  adj_fill_rand(c->luj, 3 * P, 48, c->stream);
  for (int sgn = 1; sgn >= -1; sgn -= 2) {
    for (int q = 0; q < 2; ++q) adj_axpy(a_[q], a0[q], va[q], sgn * hstep, slots, c->stream);
    for (int q = 0; q < 5; ++q) adj_axpy(b_[q], b0[q], vb[q], sgn * hstep, slots, c->stream);
    fast::deposit2d(d, c->stream);
    adj_dot(d.uj, c->luj, 3 * P, dots + (sgn > 0 ? 0 : 1), c->stream);
  }
  adj_copy_parts(A0, d.A, slots, c->stream);
  adj_copy_parts(B0, d.B, slots, c->stream);
  adj_zero_parts(c->lA, slots, c->stream);
  adj_zero_parts(c->lB, slots, c->stream);
  adj_deposit_only(d, c->luj, c->lA, c->lB, c->adj_fp32 ? c->adj_f32 : nullptr, c->stream);
  double* la[2] = {c->lA.x, c->lA.y};
  double* lb[5] = {c->lB.x, c->lB.y, c->lB.ux, c->lB.uy, c->lB.uz};
  for (int q = 0; q < 2; ++q) adj_dot(va[q], la[q], slots, dots + 2, c->stream);
  for (int q = 0; q < 5; ++q) adj_dot(vb[q], lb[q], slots, dots + 2, c->stream);
  double h[3];
  CK(cudaMemcpyAsync(h, dots, 3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  out[0] = (h[0] - h[1]) * 0.5 / hstep;
  out[1] = h[2];
  return finish(c);
}

// central difference of <lJ, J(A, push(A, uf))> along a random direction of the fields against
// push_F^T deposit_B^T lJ: out2 = {difference, adjoint}.  The fields are restored.
int wpic_adjoint_chaincheck(wpic_ctx* c, double hstep, double* out) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mixed || !out || !(hstep > 0)) return WPIC_BAD_ARGUMENT;
  Dev2D& d = c->d;
  int st = adj_prepare(c, 0);
  if (st) return st;
  const size_t P = d.g.fplane, slots = (size_t)d.nrowjob * d.cap;
  if ((st = chk_scratch(c, false, true))) return st;
  double *const dots = c->chk_dots, *const f0 = c->chk_f0, *const v = c->chk_v, *const lj = c->chk_lj;
  cudaMemsetAsync(dots, 0, 4 * sizeof(double), c->stream);
  cudaMemcpyAsync(f0, d.uf, 6 * P * 8, cudaMemcpyDeviceToDevice, c->stream);
  adj_fill_rand(v, 6 * P, 51, c->stream);
  adj_fill_rand(lj, 3 * P, 52, c->stream);
  for (int sgn = 1; sgn >= -1; sgn -= 2) {
    adj_axpy(d.uf, f0, v, sgn * hstep, 6 * P, c->stream);
    fast::push2d(d, c->stream);
    fast::deposit2d(d, c->stream);
    adj_dot(d.uj, lj, 3 * P, dots + (sgn > 0 ? 0 : 1), c->stream);
  }
  cudaMemcpyAsync(d.uf, f0, 6 * P * 8, cudaMemcpyDeviceToDevice, c->stream);
  fast::push2d(d, c->stream);
  cudaMemsetAsync(c->luf, 0, 6 * P * 8, c->stream);
  adj_zero_parts(c->lA, slots, c->stream);
  adj_zero_parts(c->lB, slots, c->stream);
  adj_particles(d, lj, c->lA, c->lB, c->tmpc, c->ltmp, c->luf, c->adj_fp32 ? c->adj_f32 : nullptr, c->stream);
  adj_dot(v, c->luf, 6 * P, dots + 2, c->stream);
  double h[3];
  CK(cudaMemcpyAsync(h, dots, 3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  out[0] = (h[0] - h[1]) * 0.5 / hstep;
  out[1] = h[2];
  return finish(c);
}

// Arithmetic of the adjoint's per-particle sweeps: WPIC_FP64 (or WPIC_FP64_EXACT) for FP64,
// WPIC_MIXED for FP32 push and deposit reverses along the recorded FP64 trajectory; the field
// adjoint, the adjoint CG and every accumulation stay FP64.
int wpic_adjoint_precision(wpic_ctx* c, int precision) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (precision != WPIC_FP64 && precision != WPIC_FP64_EXACT && precision != WPIC_MIXED) return WPIC_BAD_ARGUMENT;
  c->adj_fp32 = precision == WPIC_MIXED;
  return WPIC_OK;
}

int wpic_adjoint_keep_fields(wpic_ctx* c, int keep) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (keep != 0 && keep != 1) return WPIC_BAD_ARGUMENT;
  c->adj_keep_fields = keep == 1;
  if (!keep && c->adj_fields) {  // give the store back; a recorded run is then recomputed in full
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaFree(c->adj_fields));
    c->adj_fields = nullptr;
    c->adj_fields_slots = 0;
    c->adj_nfield = 0;
  }
  return WPIC_OK;
}

// Forward half of the adjoint: nsteps steps from the current state, keeping the particle and
// field state at every segment start (every K steps) and at the end.
int wpic_adjoint_record(wpic_ctx* c, int nsteps, int every) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mixed || c->d.ph.bc != BC_PERIODIC || c->pusher != WPIC_PUSH_BORIS || nsteps < 1 || every < 1)
    return WPIC_BAD_ARGUMENT;
  const int nseg = (nsteps + every - 1) / every;
  c->adj_nsteps = 0;
  int st = adj_prepare(c, nseg + every + 1);
  if (st) return st;
  // the last segment keeps its step states as it runs: the reverse sweep starts on it
  // without recomputing it; the field state before each step 1 .. last0 - 1 goes to the
  // field store (the other segments' recompute replays it)
  const int last0 = (nseg - 1) * every;
  c->adj_last_kept = false;
  if ((st = adj_field_store(c, last0 - 1))) return st;
  for (int k = 0; k < nsteps; ++k) {
    if (k % every == 0) adj_save(c, c->adj_states[k / every]);
    if (k >= last0) {
      wpic_ctx::AdjState& S = c->adj_states[nseg + (k - last0)];
      adj_save(c, S);
      S.has_step = false;
      if (k + 1 < nsteps) {  // the segment's last step is pushed and sorted again by adj_step
        if ((st = adj_alloc_step(c, S)) || (st = adj_forward_step(c, S))) return st;
        continue;
      }
    }
    if ((st = one_step(c))) return st;
    if (k + 1 <= c->adj_nfield) adj_field_slot(c, k + 1, true);
  }
  adj_save(c, c->adj_states[nseg + every]);
  if ((st = finish(c))) return st;
  c->adj_last_kept = true;
  c->adj_nsteps = nsteps;
  c->adj_every = every;
  return WPIC_OK;
}

// Reverse half: given the gradient of a scalar with respect to the recorded final fields,
// the gradients with respect to the recorded initial particles (reference layout of up, ids
// in the last slot) and fields (layout of uf).  Each segment is recomputed from its start,
// its step states kept, and the steps are reversed.  Leaves the recorded final state.
int wpic_adjoint_reverse(wpic_ctx* c, const double* lam_uf_final, double* lam_up0, double* lam_uf0) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (!lam_uf_final || !lam_up0 || !lam_uf0) return WPIC_BAD_ARGUMENT;
  if (c->adj_nsteps < 1) return WPIC_BAD_ARGUMENT;  // nothing recorded
  Dev2D& d = c->d;
  const int nsteps = c->adj_nsteps, every = c->adj_every;
  const int nseg = (nsteps + every - 1) / every;
  int fixed_saved[3];
  for (int l = 0; l < 3; ++l) fixed_saved[l] = c->cg_fixed[l];
  auto ckpt = [&](int k) -> wpic_ctx::AdjState& { return c->adj_states[k]; };
  auto step_state = [&](int k) -> wpic_ctx::AdjState& { return c->adj_states[nseg + k]; };
  wpic_ctx::AdjState& fin = c->adj_states[nseg + every];
  int st = put_field(c, lam_uf_final, c->luf, 6);  // the seed: the final fields' adjoint
  if (st) return st;
  adj_zero_parts(c->lA, (size_t)d.nrowjob * d.cap, c->stream);
  for (int l = 0; l < 3; ++l) c->cg_fixed[l] = -1;  // adjoint solves: the tolerance rule
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int s0 = seg * every, s1 = std::min(nsteps, s0 + every);
    const bool kept = seg == nseg - 1 && c->adj_last_kept;
    if (!kept) adj_load(c, ckpt(seg));
    for (int k = s0; k < s1 && !kept; ++k) {
      wpic_ctx::AdjState& S = step_state(k - s0);
      adj_save(c, S);
      S.has_step = false;
      if (k + 1 < s1) {  // the segment's last step is pushed and sorted again by adj_step
        const int replay = k + 1 <= c->adj_nfield ? k + 1 : 0;
        if ((st = adj_alloc_step(c, S)) || (st = adj_forward_step(c, S, replay))) break;
      }
    }
    if (st) break;
    for (int k = s1 - 1; k >= s0; --k) {
      adj_load(c, step_state(k - s0));
      if ((st = adj_step(c, &step_state(k - s0)))) break;
    }
    if (st) break;
    if ((st = finish(c))) break;
    if (seg < nseg - 1) c->adj_last_kept = false;  // the step states now hold this segment
  }
  for (int l = 0; l < 3; ++l) c->cg_fixed[l] = fixed_saved[l];
  if (st) return st;
  // d holds the initial state: the particle gradient in its slot order, with its ids
  const int ndim = c->prm.ndim, nph = c->prm.np;
  const size_t row_bytes = (size_t)ndim * nph * sizeof(double);
  if ((st = ensure_staging(c, (size_t)d.nrowjob * row_bytes))) return st;
  Parts64 G = c->lA;
  G.id = d.A.id;
  soa_to_aos2d(d, c->staging, ndim, nph, 0, d.nrowjob, G, c->stream);
  CK(cudaMemcpyAsync(lam_up0, c->staging, (size_t)d.nrowjob * row_bytes, cudaMemcpyDeviceToHost, c->stream));
  if ((st = finish(c))) return st;
  if ((st = get_field(c, lam_uf0, c->luf, 6))) return st;
  adj_load(c, fin);
  return finish(c);
}

int wpic_adjoint(wpic_ctx* c, int nsteps, int every, const double* lam_uf_final, double* lam_up0,
                 double* lam_uf0) {
  if (!lam_uf_final || !lam_up0 || !lam_uf0) return WPIC_BAD_ARGUMENT;
  int st = wpic_adjoint_record(c, nsteps, every);
  return st ? st : wpic_adjoint_reverse(c, lam_uf_final, lam_up0, lam_uf0);
}

int wpic_put_fields(wpic_ctx* c, const double* uf) { return c ? put_field(c, uf, c->d.uf, 6) : WPIC_NOT_INITIALISED; }
int wpic_get_fields(wpic_ctx* c, double* uf) { return c ? get_field(c, uf, c->d.uf, 6) : WPIC_NOT_INITIALISED; }
int wpic_put_df(wpic_ctx* c, const double* df) { return c ? put_field(c, df, c->d.df, 6) : WPIC_NOT_INITIALISED; }
int wpic_get_df(wpic_ctx* c, double* df) { return c ? get_field(c, df, c->d.df, 6) : WPIC_NOT_INITIALISED; }
int wpic_get_uj(wpic_ctx* c, double* uj) { return c ? get_field(c, uj, c->d.uj, 3) : WPIC_NOT_INITIALISED; }

namespace {
// The staged calls on a mixed context.  The mixed step pushes, deposits, applies the x
// boundary, moves the cell-leavers into their columns and solves the fields in one sequence
// (mixed_step), so the drivers' calls map onto it: particle__solv asks for the push,
// field__fdtd_i runs the whole step, and particle_x, particle_y and sort__bucket find their
// work done.  Both driver orders are accepted (Weibel: push, field, particle_x; reconnection:
// push, particle_x, field); the shock driver's injection call between the push and the field
// solve sets the u0 the step uses.
int mix_request_push(wpic_ctx* c, int pusher) {
  if (c->mix_pending) return WPIC_BAD_ARGUMENT;  // a second push before the field solve
  c->mix_pending = true;
  c->mix_pending_pusher = pusher;
  return WPIC_OK;
}

int mix_run_requested(wpic_ctx* c) {
  if (!c->mix_pending) return WPIC_BAD_ARGUMENT;  // the field solve cannot run without its push
  c->mix_pending = false;
  const int saved = c->pusher;
  c->pusher = c->mix_pending_pusher;
  const int st = one_step(c);
  c->pusher = saved;
  const int st2 = finish(c);
  return st ? st : st2;
}
}  // namespace

int wpic_particle_solv(wpic_ctx* c) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mixed) return mix_request_push(c, WPIC_PUSH_BORIS);
  do_push(c);
  return finish(c);
}

int wpic_particle_solv_vay(wpic_ctx* c) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mixed) return mix_request_push(c, WPIC_PUSH_VAY);
  FP(push_vay2d, c->d, c->stream);
  return finish(c);
}

int wpic_set_pusher(wpic_ctx* c, int pusher) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (pusher != WPIC_PUSH_BORIS && pusher != WPIC_PUSH_VAY) return WPIC_BAD_ARGUMENT;
  c->pusher = pusher;
  return WPIC_OK;
}

int wpic_set_window(wpic_ctx* c, int nxs, int nxe) {
  if (!c) return WPIC_NOT_INITIALISED;
  const int nxge = c->d.g.nxgs + c->d.g.nx - 1;
  if (nxs < c->d.g.nxgs || nxe > nxge || nxe - nxs < 3) return WPIC_BAD_ARGUMENT;
  const bool full = nxs == c->d.g.nxgs && nxe == nxge;
  if (!full && (c->d.ph.bc == BC_PERIODIC || (c->mixed && c->d.ph.bc != BC_SHOCK))) return WPIC_BAD_ARGUMENT;
  c->d.g.wx0 = nxs - c->d.g.nxgs;
  c->d.g.wx1 = nxe - c->d.g.nxgs;
  return WPIC_OK;
}

int wpic_set_injection(wpic_ctx* c, double u0) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (!(u0 == u0)) return WPIC_BAD_ARGUMENT;
  c->u0 = u0;
  return WPIC_OK;
}

int wpic_bc_injection(wpic_ctx* c, double u0) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->d.ph.bc != BC_SHOCK || !(u0 == u0)) return WPIC_BAD_ARGUMENT;
  if (c->mixed) {  // between the requested push and the field solve: the step's u0
    if (!c->mix_pending) return WPIC_BAD_ARGUMENT;
    c->u0 = u0;
    return WPIC_OK;
  }
  do_injection(c, u0);
  return finish(c);
}

int wpic_field_fdtd_i(wpic_ctx* c) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mixed) return mix_run_requested(c);
  int st = do_field(c);
  int st2 = finish(c);
  return st ? st : st2;
}

int wpic_ele_cur(wpic_ctx* c) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mixed) return WPIC_BAD_ARGUMENT;
  do_ele_cur(c);
  return finish(c);
}

int wpic_bc_particle_x(wpic_ctx* c) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mixed) return WPIC_OK;  // inside the mixed step, before or after its field solve
  do_particle_x(c);
  return finish(c);
}

int wpic_bc_particle_y(wpic_ctx* c) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mixed) return c->mix_pending ? WPIC_BAD_ARGUMENT : WPIC_OK;  // done by the mixed step
  int st = ensure_C(c);
  if (st) return st;
  Dev2D& d = c->d;
  stage_begin(c, SG_PBC);
  migrate_scan2d(d, d.B, c->stream);
  migrate_plan2d(d, c->stream);
  gather2d(d, d.B, d.C, d.slist, d.np2new, c->stream);
  CK(cudaMemcpyAsync(d.np2, d.np2new, sizeof(int) * d.nrowjob, cudaMemcpyDeviceToDevice, c->stream));
  stage_end(c, SG_PBC, 3);
  const Parts64 t = d.B;
  d.B = d.C;
  d.C = t;
  return finish(c);
}

int wpic_sort_bucket(wpic_ctx* c) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mixed) return c->mix_pending ? WPIC_BAD_ARGUMENT : WPIC_OK;  // done by the mixed step
  Dev2D& d = c->d;
  stage_begin(c, SG_SORT);
  sort_rank2d(d, d.B, nullptr, c->stream);
  gather2d(d, d.B, d.A, d.map, d.np2, c->stream);
  stage_end(c, SG_SORT, 2);
  return finish(c);
}

int wpic_step(wpic_ctx* c, int nsteps) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mix_pending) return WPIC_BAD_ARGUMENT;  // a requested push waits for field__fdtd_i
  for (int it = 0; it < nsteps; ++it) {
    int st = one_step(c);
    int st2 = finish(c);
    if (st) return st;
    if (st2) return st2;
  }
  return WPIC_OK;
}

int wpic_energy(wpic_ctx* c, double* out) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (!out) return WPIC_BAD_ARGUMENT;
  if (c->mixed) mix_energy2d(c->d, c->stream);
  else FP(energy2d, c->d, c->stream);
  double h[4];
  CK(cudaMemcpyAsync(h, c->d.red_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  int st = finish(c);
  if (st) return st;
  const int nsp = c->prm.nsp;
  for (int k = 0; k < nsp; ++k) out[k] = h[k];
  out[nsp] = h[2] / (8 * c->d.ph.pi);
  out[nsp + 1] = h[3] / (8 * c->d.ph.pi);
  return WPIC_OK;
}

namespace {
size_t mom_count(const wpic_ctx* c) { return 7 * (size_t)(c->d.g.nx + 2) * (c->d.g.ny + 2) * c->d.ph.nsp; }

int ensure_mom(wpic_ctx* c) {
  if (c->mom) return WPIC_OK;
  return dalloc(c, &c->mom, mom_count(c));
}

int copy_mom(wpic_ctx* c, double* out) {
  if (!out) return WPIC_OK;
  CK(cudaMemcpyAsync(out, c->mom, mom_count(c) * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  return WPIC_OK;
}
}  // namespace

// On a mixed context the diagnostic block's three calls map onto the mixed moments kernel,
// which pushes the half step in FP32 without touching the particle state and folds the
// ghost nodes: mom_calc__accl has nothing to write, mom_calc__nvt (after it, from gp)
// computes the folded moments, bc__mom finds them folded.
int wpic_mom_calc_accl(wpic_ctx* c) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (c->mixed) return c->mix_pending ? WPIC_BAD_ARGUMENT : WPIC_OK;
  FP(mom_accl2d, c->d, c->stream);
  return finish(c);
}

int wpic_mom_calc_nvt(wpic_ctx* c, int from_gp) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (from_gp != 0 && from_gp != 1) return WPIC_BAD_ARGUMENT;
  if (c->mixed && (from_gp != 1 || c->mix_pending)) return WPIC_BAD_ARGUMENT;
  int st = ensure_mom(c);
  if (st) return st;
  if (c->mixed) mix_moments2d(c->d, c->mom, c->stream);
  else FP(mom_nvt2d, c->d, from_gp ? c->d.B : c->d.A, c->mom, c->stream);
  return finish(c);
}

int wpic_bc_mom(wpic_ctx* c) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (!c->mom) return WPIC_BAD_ARGUMENT;
  if (c->mixed) return WPIC_OK;  // the mixed moments come folded
  bc_mom2d(c->d, c->mom, c->stream);
  return finish(c);
}

int wpic_get_mom(wpic_ctx* c, double* mom) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (!c->mom || !mom) return WPIC_BAD_ARGUMENT;
  int st = copy_mom(c, mom);
  if (st) return st;
  return finish(c);
}

int wpic_moments(wpic_ctx* c, double* mom) {
  if (!c) return WPIC_NOT_INITIALISED;
  int st = ensure_mom(c);
  if (st) return st;
  if (c->mixed) {
    mix_moments2d(c->d, c->mom, c->stream);
  } else {
    FP(mom_accl2d, c->d, c->stream);
    FP(mom_nvt2d, c->d, c->d.B, c->mom, c->stream);
    bc_mom2d(c->d, c->mom, c->stream);
  }
  if ((st = copy_mom(c, mom))) return st;
  return finish(c);
}

int wpic_cg_control(wpic_ctx* c, const int* fixed3, int ite_max) {
  if (!c) return WPIC_NOT_INITIALISED;
  for (int l = 0; l < 3; ++l) c->cg_fixed[l] = fixed3 ? fixed3[l] : -1;
  c->d.ite_max = ite_max > 0 ? ite_max : 100;
  return WPIC_OK;
}

int wpic_cg_tolerance(wpic_ctx* c, double rtol, int ite_max) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (!(rtol > 0.0) || rtol >= 1.0 || ite_max < 1) return WPIC_BAD_ARGUMENT;
  c->d.cg_rtol = rtol;
  c->d.ite_max = ite_max;
  return WPIC_OK;
}

int wpic_cg_iters(wpic_ctx* c, int* out3) {
  if (!c) return WPIC_NOT_INITIALISED;
  if (!out3) return WPIC_BAD_ARGUMENT;
  for (int l = 0; l < 3; ++l) out3[l] = c->cg_iters[l];
  return WPIC_OK;
}

int wpic_load_weibel_2d(wpic_ctx* c, int ppc, uint64_t seed, double drift, int drift_axis, double u_thi,
                        double u_the, const double* b0) {
  if (!c) return WPIC_NOT_INITIALISED;
  Dev2D& d = c->d;
  if (drift_axis < 0 || drift_axis > 2 || ppc < 1) return WPIC_BAD_ARGUMENT;
  if (c->mixed) {
    const int dep = mix_initial_depth(ppc, c->prm.c * c->prm.delt / c->prm.delx);
    int st = mix_set_layout(c, std::vector<int>(d.m.nbin, dep), false);
    if (st) return st;
    mix_load_weibel2d(d, ppc, seed, drift, drift_axis, u_thi, u_the, c->stream);
  } else {
    if ((long long)ppc * d.g.nx > d.cap) return WPIC_CAPACITY;
    load_weibel2d_ppc(d, ppc, seed, drift, drift_axis, u_thi, u_the, c->stream);
  }
  const size_t fplane = d.g.fplane;
  CK(cudaMemsetAsync(d.uf, 0, 6 * fplane * sizeof(double), c->stream));
  CK(cudaMemsetAsync(d.df, 0, 6 * fplane * sizeof(double), c->stream));
  CK(cudaMemsetAsync(d.uj, 0, 3 * fplane * sizeof(double), c->stream));
  if (b0) {
    std::vector<double> plane(fplane);
    for (int k = 0; k < 3; ++k) {
      if (b0[k] == 0.0) continue;
      for (size_t i = 0; i < fplane; ++i) plane[i] = b0[k];
      CK(cudaMemcpyAsync(d.uf + k * fplane, plane.data(), fplane * sizeof(double), cudaMemcpyHostToDevice,
                         c->stream));
      CK(cudaStreamSynchronize(c->stream));
    }
  }
  return finish(c);
}

int wpic_timing_enable(wpic_ctx* c, int enable) {
  if (!c) return WPIC_NOT_INITIALISED;
  cudaStreamSynchronize(c->stream);
  stage_collect(c);
  c->timing = enable != 0;
  for (int s = 0; s < SG_COUNT; ++s) {
    c->stage_ms[s] = 0.0;
    c->stage_launches[s] = 0;
    c->pending[s] = false;
  }
  return WPIC_OK;
}

int wpic_timing_get(wpic_ctx* c, double* ms, long long* launches, int n) {
  if (!c) return WPIC_NOT_INITIALISED;
  cudaStreamSynchronize(c->stream);
  stage_collect(c);
  for (int s = 0; s < n && s < SG_COUNT; ++s) {
    if (ms) ms[s] = c->stage_ms[s];
    if (launches) launches[s] = c->stage_launches[s];
  }
  return WPIC_OK;
}

const char* wpic_stage_name(int s) { return (s >= 0 && s < SG_COUNT) ? kStageNames[s] : "?"; }
int wpic_num_stages(void) { return SG_COUNT; }

int wpic_host_register(void* ptr, size_t bytes) {
  if (!ptr || !bytes) return WPIC_BAD_ARGUMENT;
  return cuda_status(cudaHostRegister(ptr, bytes, cudaHostRegisterMapped));
}

int wpic_host_unregister(void* ptr) {
  if (!ptr) return WPIC_BAD_ARGUMENT;
  return cuda_status(cudaHostUnregister(ptr));
}

int wpic_synchronize(wpic_ctx* c) {
  if (!c) return WPIC_NOT_INITIALISED;
  return finish(c);
}

long long wpic_num_particles(wpic_ctx* c) {
  if (!c) return -1;
  const bool mx = c->mixed;
  std::vector<int> h(mx ? (size_t)c->d.m.nbin * MIX_TC : (size_t)c->d.nrowjob);
  if (cudaMemcpyAsync(h.data(), mx ? c->d.m.cnt : c->d.np2, sizeof(int) * h.size(), cudaMemcpyDeviceToHost,
                      c->stream) !=
      cudaSuccess)
    return -1;
  cudaStreamSynchronize(c->stream);
  long long n = 0;
  for (int v : h) n += v;
  return n;
}

const char* wpic_status_string(int s) {
  switch (s) {
    case WPIC_OK: return "ok";
    case WPIC_CG_NOT_CONVERGED: return "CG did not converge within ite_max iterations";
    case WPIC_CAPACITY: return "particle capacity of a row exceeded";
    case WPIC_OUT_OF_RANGE: return "particle outside the domain";
    case WPIC_MOVED_TOO_FAR: return "particle moved more than one cell in one step";
    case WPIC_NONFINITE: return "non-finite value";
    case WPIC_BAD_ARGUMENT: return "bad argument";
    case WPIC_CUDA_ERROR: return "CUDA error";
    case WPIC_NOT_INITIALISED: return "context not initialised";
    case WPIC_STAGING_TIMEOUT: return "bulk copy into shared memory timed out (finalise the context)";
    default: return "unknown status";
  }
}

}  // extern "C"
