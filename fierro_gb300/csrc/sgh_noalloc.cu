// Energy tallies that allocate nothing.
//
// Some callers of this library cannot call cudaMalloc when they want the
// tallies: a hydrocode driver that captures its whole time step, diagnostics
// included, into a CUDA graph may not allocate while the capture is open, and a
// code that hands all device memory to its own arena at start-up has no
// allocation budget left for a library's temporaries.  For them
// fierro_energy_tally_noalloc computes IE = sum M e and KE = 1/2 sum m |v|^2
// (the tallies of the SGH cycle loop) over device arrays the caller owns, with
// the per-block partial sums kept in the file-scope array below instead of
// memory the library allocates.
//
// The array is 8 KiB (2 x 512 doubles) and lives on every GPU that loads the
// library until the process exits.  Every call shares it: calls that overlap on
// the GPU (different streams without ordering) race on it.  Each call writes
// every partial it later reads, so the previous call's contents never need
// clearing.
#include <cstdint>
#include <mutex>

#include <cuda.h>
#include <cuda_runtime.h>

#include "fierro_sgh.h"
#include "sgh_internal.h"

namespace {

constexpr int kTallyBlocks = 512;
constexpr int kTallyThreads = 256;
// Largest array length a call accepts: the kernels index with 32-bit integers
// and stride by the whole grid, so counts stay below 2^31 - grid size.
constexpr int64_t kTallyMaxLength = (int64_t)1 << 30;

static __device__ __align__(256) double g_tally_scratch[2 * kTallyBlocks];

__global__ void __launch_bounds__(kTallyThreads)
k_tally_part(const double* __restrict__ mass, const double* __restrict__ sie, int ne,
             const double* __restrict__ node_mass, const double* __restrict__ u,
             const double* __restrict__ v, const double* __restrict__ w, int nn, double* part) {
  __shared__ double sh[2][kTallyThreads];
  double ie = 0.0, ke = 0.0;
  const int stride = gridDim.x * blockDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ne; i += stride) ie += mass[i] * sie[i];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += stride) {
    double k = 0;
    k += u[i] * u[i];
    k += v[i] * v[i];
    k += w[i] * w[i];
    ke += node_mass[i] * k;
  }
  sh[0][threadIdx.x] = ie;
  sh[1][threadIdx.x] = ke;
  __syncthreads();
  for (int s = kTallyThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + s];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[blockIdx.x] = sh[0][0];
    part[gridDim.x + blockIdx.x] = sh[1][0];
  }
}

__global__ void k_tally_final(const double* part, int nblocks, double* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double ie = 0.0, ke = 0.0;
  for (int b = 0; b < nblocks; ++b) {
    ie += part[b];
    ke += part[nblocks + b];
  }
  out[0] = ie;
  out[1] = 0.5 * ke;
}

// The scratch array's device address belongs to the CUDA context that loaded
// this module, not to the device: after cudaDeviceReset (or any other teardown
// and re-creation of the primary context) the module is loaded again, possibly
// at another address, and a second context on the same device (cuCtxCreate)
// holds its own copy of the array.  The address is therefore cached per
// context, under the driver's process-unique context id, and looked up again
// for a context not seen before.  The lookup (cudaGetSymbolAddress, which may
// load the module) happens on the first call in each context; that call should
// come before any stream capture in that context.
constexpr int kMaxContexts = 64;

struct ScratchEntry {
  unsigned long long ctx_id;
  double* addr;
};

std::mutex g_setup_mutex;
ScratchEntry g_scratch[kMaxContexts] = {};
int g_scratch_used = 0, g_scratch_next = 0;

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

// The driver's cuCtxGetCurrent / cuCtxGetId, through the runtime's entry-point
// query (the library does not link libcuda itself).  Called with the mutex held.
int driver_entry_points() {
  if (g_ctx_get_current && g_ctx_get_id) return FIERRO_OK;
  void* f1 = nullptr;
  void* f2 = nullptr;
  cudaDriverEntryPointQueryResult q1{}, q2{};
  cudaError_t e1 = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
  cudaError_t e2 = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
  if (e1 != cudaSuccess || e2 != cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
      q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
    return fierro::set_error(FIERRO_ECUDA, "energy tally: driver entry points cuCtxGetCurrent/cuCtxGetId unavailable");
  g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
  g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
  return FIERRO_OK;
}

// Device address of g_tally_scratch in the current context.  In host code the
// array's name is only a host-side stand-in, so the kernels are always given
// this address.
int scratch_address(double** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  int rc = driver_entry_points();
  if (rc) return rc;
  CUcontext ctx = nullptr;
  if (g_ctx_get_current(&ctx) != CUDA_SUCCESS)
    return fierro::set_error(FIERRO_ECUDA, "energy tally: cuCtxGetCurrent failed");
  void* p = nullptr;
  if (!ctx) {
    // no context is current on this thread yet: the runtime call below makes
    // the current device's primary context current
    cudaError_t err = cudaGetSymbolAddress(&p, g_tally_scratch);
    if (err != cudaSuccess || !p)
      return fierro::set_error(FIERRO_ECUDA, "cudaGetSymbolAddress(tally scratch): %s", cudaGetErrorString(err));
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx)
      return fierro::set_error(FIERRO_ECUDA, "energy tally: no current CUDA context");
  }
  unsigned long long id = 0;
  if (g_ctx_get_id(ctx, &id) != CUDA_SUCCESS) return fierro::set_error(FIERRO_ECUDA, "energy tally: cuCtxGetId failed");
  for (int i = 0; i < g_scratch_used; ++i)
    if (g_scratch[i].ctx_id == id) {
      *out = g_scratch[i].addr;
      return FIERRO_OK;
    }
  if (!p) {
    cudaError_t err = cudaGetSymbolAddress(&p, g_tally_scratch);
    if (err != cudaSuccess || !p)
      return fierro::set_error(FIERRO_ECUDA, "cudaGetSymbolAddress(tally scratch): %s", cudaGetErrorString(err));
  }
  // context ids are never reused within a process, so an entry of a destroyed
  // context is only ever dead weight: the oldest entry makes room when full
  ScratchEntry& e = g_scratch_used < kMaxContexts ? g_scratch[g_scratch_used++] : g_scratch[g_scratch_next++];
  if (g_scratch_next == kMaxContexts) g_scratch_next = 0;
  e.ctx_id = id;
  e.addr = static_cast<double*>(p);
  *out = e.addr;
  return FIERRO_OK;
}

}  // namespace

extern "C" int fierro_energy_tally_noalloc(const double* elem_mass, const double* elem_sie, int64_t num_elems,
                                           const double* node_mass, const double* node_u, const double* node_v,
                                           const double* node_w, int64_t num_nodes, double* ie_ke, void* stream) {
  fierro::clear_error();
  if (num_elems < 0 || num_nodes < 0)
    return fierro::set_error(FIERRO_EINVAL, "energy tally: negative length");
  if (num_elems > kTallyMaxLength || num_nodes > kTallyMaxLength)
    return fierro::set_error(FIERRO_EINVAL,
                             "energy tally: %lld elements / %lld nodes exceed the maximum of %lld per array",
                             (long long)num_elems, (long long)num_nodes, (long long)kTallyMaxLength);
  if (!ie_ke || (num_elems > 0 && (!elem_mass || !elem_sie)) ||
      (num_nodes > 0 && (!node_mass || !node_u || !node_v || !node_w)))
    return fierro::set_error(FIERRO_EINVAL, "energy tally: NULL array");
  double* scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_tally_part<<<kTallyBlocks, kTallyThreads, 0, s>>>(elem_mass, elem_sie, (int)num_elems, node_mass, node_u,
                                                      node_v, node_w, (int)num_nodes, scratch);
  k_tally_final<<<1, 32, 0, s>>>(scratch, kTallyBlocks, ie_ke);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return fierro::set_error(FIERRO_ECUDA, "energy tally launch: %s", cudaGetErrorString(err));
  return FIERRO_OK;
}
