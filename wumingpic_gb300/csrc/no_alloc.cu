// wpic_energy_noalloc: the energy_history sums for callers that cannot allocate
// device memory.
//
// wpic_energy needs a context, and a context allocates the whole device state
// of a run.  Some callers cannot do that at the point where they want the
// diagnostic: a driver whose particle and field arrays already live on the
// device under another runtime's allocator (OpenACC or CUDA Fortran data
// regions, a framework's memory pool) and that must not add allocations of its
// own; a time-step loop where a cudaMalloc would synchronise the device and
// stall the step; or a run sized to fill HBM, where no headroom is left for a
// late allocation.  This entry point takes the caller's device arrays and
// output, and keeps its only scratch -- the per-row partial sums that make the
// reduction order fixed -- in a file-scope __device__ array of fixed size,
// which every GPU that loads this library holds until the process exits.
//
// The scratch is shared by all calls and keeps the last call's contents; every
// slot a call reads is first written by that same call, so nothing needs to be
// cleared.  Calls that overlap on the GPU (different streams, or several host
// threads on one device) race on the scratch and must be serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>

#include "wumingpic_gb300.h"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

// [0, MAX): kinetic partial per (species, row); [MAX, 2 MAX): sum E^2 per row; [2 MAX, 3 MAX): sum B^2 per row
static __device__ __align__(256) double g_energy_scratch[3 * WPIC_NOALLOC_MAX_ROWS];

void* g_scratch_addr[kMaxDevices] = {};
std::mutex g_setup_mutex;

// Device address of the scratch array for the current device, looked up once per device.
// The cached address belongs to the context that was current at the look-up: after a
// cudaDeviceReset the module is loaded again in a new context and the array may move, so
// the entry point is not for use after a device reset (the header says so).
int scratch_address(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return WPIC_CUDA_ERROR;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_energy_scratch) != cudaSuccess || !p) return WPIC_CUDA_ERROR;
    g_scratch_addr[dev] = p;
  }
  *out = static_cast<double*>(g_scratch_addr[dev]);
  return WPIC_OK;
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + w];
    __syncthreads();
  }
  return sh[0];
}

struct Args {
  const double* up;
  const int* np2;
  const double* uf;
  int ndim, np, nx, ny, nsp;
  double r[2];
  double c;
  double* out;
  double* scratch;
};

// one block per (species, row): sum of r (gamma - 1) over the row's particles
__global__ void __launch_bounds__(kThreads) k_kinetic_rows(Args a) {
  __shared__ double sh[kThreads];
  const int row = blockIdx.x;  // isp * ny + jj, the reference's row order of up(ndim, np, ny, nsp)
  const int isp = row / a.ny;
  const int n = a.np2[row];
  const double* base = a.up + (size_t)row * a.np * a.ndim;
  const double rr = a.r[isp], c2 = a.c * a.c;
  double v = 0.0;
  for (int s = threadIdx.x; s < n && s < a.np; s += kThreads) {
    const double* u = base + (size_t)s * a.ndim;
    const double u2 = u[2] * u[2] + u[3] * u[3] + u[4] * u[4];
    v = v + rr * (sqrt(1 + u2 / c2) - 1);
  }
  v = block_sum(v, sh);
  if (threadIdx.x == 0) a.scratch[row] = v;
}

// one block per interior row: sums of E^2 and B^2 of uf(6, nx+4, ny+4)
__global__ void __launch_bounds__(kThreads) k_field_rows(Args a) {
  __shared__ double sh[kThreads];
  const int jj = blockIdx.x;
  const size_t pitch = (size_t)a.nx + 4;
  const double* row = a.uf + 6 * ((size_t)(jj + 2) * pitch + 2);
  double e = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < a.nx; i += kThreads) {
    const double* f = row + 6 * (size_t)i;
    b = b + f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    e = e + f[3] * f[3] + f[4] * f[4] + f[5] * f[5];
  }
  e = block_sum(e, sh);
  __syncthreads();
  b = block_sum(b, sh);
  if (threadIdx.x == 0) {
    a.scratch[WPIC_NOALLOC_MAX_ROWS + jj] = e;
    a.scratch[2 * WPIC_NOALLOC_MAX_ROWS + jj] = b;
  }
}

// one block: the row partials in a fixed order -> out[0..nsp-1], E^2/8pi, B^2/8pi
__global__ void __launch_bounds__(kThreads) k_finish(Args a) {
  __shared__ double sh[kThreads];
  const double pi = 3.141592653589793;
  for (int isp = 0; isp < a.nsp; ++isp) {
    double v = 0.0;
    for (int k = threadIdx.x; k < a.ny; k += kThreads) v = v + a.scratch[isp * a.ny + k];
    v = block_sum(v, sh);
    if (threadIdx.x == 0) a.out[isp] = v;
    __syncthreads();
  }
  double e = 0.0, b = 0.0;
  for (int k = threadIdx.x; k < a.ny; k += kThreads) {
    e = e + a.scratch[WPIC_NOALLOC_MAX_ROWS + k];
    b = b + a.scratch[2 * WPIC_NOALLOC_MAX_ROWS + k];
  }
  e = block_sum(e, sh);
  __syncthreads();
  b = block_sum(b, sh);
  if (threadIdx.x == 0) {
    a.out[a.nsp] = e / (8 * pi);
    a.out[a.nsp + 1] = b / (8 * pi);
  }
}

}  // namespace

extern "C" int wpic_energy_noalloc(const double* up, const int* np2, const double* uf, int ndim, int np, int nx,
                                   int ny, int nsp, const double* r, double c, double* out, void* stream) {
  if (!up || !np2 || !uf || !r || !out) return WPIC_BAD_ARGUMENT;
  if (ndim < 5 || np < 1 || nx < 1 || ny < 1 || nsp < 1 || nsp > 2 || !(c > 0)) return WPIC_BAD_ARGUMENT;
  // the scratch holds one partial per (species, row) and per row: larger grids are refused
  if ((long long)ny * nsp > WPIC_NOALLOC_MAX_ROWS) return WPIC_BAD_ARGUMENT;
  double* scratch = nullptr;
  const int st = scratch_address(&scratch);
  if (st != WPIC_OK) return st;
  Args a;
  a.up = up;
  a.np2 = np2;
  a.uf = uf;
  a.ndim = ndim;
  a.np = np;
  a.nx = nx;
  a.ny = ny;
  a.nsp = nsp;
  a.r[0] = r[0];
  a.r[1] = nsp > 1 ? r[1] : 0.0;
  a.c = c;
  a.out = out;
  a.scratch = scratch;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_kinetic_rows<<<ny * nsp, kThreads, 0, s>>>(a);
  k_field_rows<<<ny, kThreads, 0, s>>>(a);
  k_finish<<<1, kThreads, 0, s>>>(a);
  return cudaGetLastError() == cudaSuccess ? WPIC_OK : WPIC_CUDA_ERROR;
}
