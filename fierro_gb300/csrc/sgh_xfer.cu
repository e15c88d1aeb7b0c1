// State transfer between the caller's host arrays (reference layouts, caller
// numbering) and the device layout (SoA, Morton numbering), done by the GPU
// reading and writing the host arrays in place.
//
// On GB300 (Grace + Blackwell over NVLink-C2C, address translation services)
// a kernel dereferences ordinary pageable host pointers: ~190 GB/s read and
// ~150 GB/s write on this machine, against ~12 GB/s for one host thread gathering
// into a staging buffer.  Threads walk the caller's numbering, so every host
// access is a coalesced stream; the permutation becomes a scatter (upload) or
// gather (download) in HBM.  Validation of the uploaded state (material ids,
// volumes, masses, and zero stress on a handle without strength materials)
// happens in the same pass and reports the first offending caller index.
#include <climits>
#include <cstdint>

#include "sgh_handle.h"
#include "sgh_xfer.h"

namespace fierro {
namespace xfer {
namespace {

constexpr int kBlock = 256;

unsigned blocks(long long n) { return (unsigned)((n + kBlock - 1) / kBlock); }

__device__ __forceinline__ void flag(XferStatus* st, int which, long long idx) {
  atomicOr(&st->flags, 1u << which);
  atomicMin(&st->first[which], idx);
}

struct NodeUp {
  int nn, dims;                        // dims: 3 (hex) or 2 (2D-RZ quads)
  const int* ext2int;
  const double *coords, *vel, *mass;  // [2][nn][dims], [2][nn][dims], [nn]
  double* x[2][3];                     // device bin b receives reference bin b ^ 1
  double* v[2][3];
  double* node_mass;
  XferStatus* st;
};

__global__ void __launch_bounds__(kBlock) k_up_nodes(const NodeUp a) {
  __shared__ double buf[kBlock * 3];
  const int j0 = blockIdx.x * kBlock;
  const int j = j0 + threadIdx.x;
  const int cnt = min(kBlock, a.nn - j0);
  const int i = j < a.nn ? a.ext2int[j] : 0;
  const int D = a.dims;
  for (int what = 0; what < 2; ++what) {
    const double* in = what == 0 ? a.coords : a.vel;
    for (int rb = 0; rb < 2; ++rb) {
      const double* src = in + ((size_t)rb * a.nn + j0) * D;
      __syncthreads();
      for (int k = threadIdx.x; k < cnt * D; k += kBlock) buf[k] = src[k];
      __syncthreads();
      if (j < a.nn)
        for (int d = 0; d < D; ++d) {
          if (what == 0) a.x[rb ^ 1][d][i] = buf[threadIdx.x * D + d];
          else a.v[rb ^ 1][d][i] = buf[threadIdx.x * D + d];
        }
    }
  }
  if (j < a.nn) {
    const double m = a.mass[j];
    a.node_mass[i] = m;
    if (!(m > 0.0)) flag(a.st, XferStatus::NODE_MASS, j);
  }
}

struct ElemUp {
  int ne, nmat, nsv;
  const int* ext2int;
  const double *sie, *den, *pres, *sspd, *vol, *mass, *statev, *div;
  const uint64_t* mat_id;
  double* d_sie[2];
  double *d_den, *d_pres, *d_sspd, *d_vol, *d_mass, *d_gamma, *d_csmin, *d_div;
  int* d_mat;
  XferStatus* st;
  // strength handles: stress [2][ne][9] -> device bins [9][ne], statev -> [nsv][ne]
  const double* stress;
  double* d_stress[2];
  double* d_statev;
};

__global__ void __launch_bounds__(kBlock) k_up_elems(const ElemUp a) {
  const int E = blockIdx.x * blockDim.x + threadIdx.x;
  if (E >= a.ne) return;
  const int e = a.ext2int[E];
  a.d_sie[1][e] = a.sie[E];                 // reference bin 0 -> device bin 1
  a.d_sie[0][e] = a.sie[(size_t)a.ne + E];  // reference bin 1 -> device bin 0
  a.d_den[e] = a.den[E];
  a.d_pres[e] = a.pres[E];
  a.d_sspd[e] = a.sspd[E];
  const double vol = a.vol[E], mass = a.mass[E];
  a.d_vol[e] = vol;
  a.d_mass[e] = mass;
  a.d_gamma[e] = a.statev[(size_t)E * a.nsv];
  a.d_csmin[e] = a.statev[(size_t)E * a.nsv + 1];
  a.d_div[e] = a.div ? a.div[E] : 0.0;
  const uint64_t mid = a.mat_id[E];
  a.d_mat[e] = mid < (uint64_t)a.nmat ? (int)mid : 0;
  if (mid >= (uint64_t)a.nmat) flag(a.st, XferStatus::MAT_ID, E);
  if (!(vol > 0.0) || !isfinite(vol)) flag(a.st, XferStatus::VOLUME, E);
  if (!(mass > 0.0)) flag(a.st, XferStatus::MASS, E);
  if (a.d_statev)
    for (int k = 0; k < a.nsv; ++k) a.d_statev[(size_t)k * a.ne + e] = a.statev[(size_t)E * a.nsv + k];
  if (a.stress) {
    // a missing stress array is a zero stress
#pragma unroll
    for (int rb = 0; rb < 2; ++rb)
#pragma unroll
      for (int k = 0; k < 9; ++k)
        a.d_stress[rb ^ 1][(size_t)k * a.ne + e] = a.stress[((size_t)rb * a.ne + E) * 9 + k];
  }
}

__global__ void __launch_bounds__(kBlock) k_zero(double* p, long long n) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    p[k] = 0.0;
}

__global__ void __launch_bounds__(kBlock) k_check_zero(const double* p, long long n, XferStatus* st) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    if (p[k] != 0.0) flag(st, XferStatus::STRESS, k);
}

// Copies buf[0, cnt) to o[0, cnt) in host memory, the whole block together, with
// 16-byte stores where o + k is 16-byte aligned (a leading and a trailing single
// store otherwise): over C2C they move the 256^3 download's node and corner-force
// rows 8 % faster than 8-byte stores (46.2 -> 42.4 ms per get_state).
__device__ __forceinline__ void store_run(double* o, const double* buf, int cnt) {
  if (reinterpret_cast<uintptr_t>(o) & 7) {
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) o[k] = buf[k];
    return;
  }
  const int head = (reinterpret_cast<uintptr_t>(o) & 15) && cnt > 0 ? 1 : 0;
  const int pairs = (cnt - head) / 2;
  double2* o2 = reinterpret_cast<double2*>(o + head);
  for (int k = threadIdx.x; k < pairs; k += blockDim.x)
    o2[k] = make_double2(buf[head + 2 * k], buf[head + 2 * k + 1]);
  if (threadIdx.x == 0 && head) o[0] = buf[0];
  if (threadIdx.x == 0 && head + 2 * pairs < cnt) o[cnt - 1] = buf[cnt - 1];
}

struct NodeDown {
  int nn, dims;
  const int* ext2int;
  double *coords, *vel, *mass;  // may be null
  const double* x[2][3];        // reference bin rb comes from device bin bins[rb]
  const double* v[2][3];
  const double* node_mass;
};

// Host stores are staged through shared memory so that each warp writes one
// contiguous run (strided 8-byte stores to host memory cost a C2C transaction each).
__global__ void __launch_bounds__(kBlock) k_down_nodes(const NodeDown a) {
  __shared__ double buf[kBlock * 3];
  const int j0 = blockIdx.x * kBlock;
  const int j = j0 + threadIdx.x;
  const int cnt = min(kBlock, a.nn - j0);
  const int i = j < a.nn ? a.ext2int[j] : 0;
  if (a.mass && j < a.nn) a.mass[j] = a.node_mass[i];
  const int D = a.dims;
  for (int what = 0; what < 2; ++what) {
    double* out = what == 0 ? a.coords : a.vel;
    if (!out) continue;
    for (int rb = 0; rb < 2; ++rb) {
      __syncthreads();
      if (j < a.nn)
        for (int d = 0; d < D; ++d) buf[threadIdx.x * D + d] = what == 0 ? a.x[rb][d][i] : a.v[rb][d][i];
      __syncthreads();
      store_run(out + ((size_t)rb * a.nn + j0) * D, buf, cnt * D);
    }
  }
}

struct ElemDown {
  int ne, nsv;
  int force_rows;  // corner-force values per element: 24 (hex) or 8 (quad)
  const int* ext2int;
  double *sie, *den, *pres, *sspd, *vol, *div, *mass, *stress, *corner_force, *statev;  // may be null
  const double* d_sie[2];  // reference bin rb
  const double *d_den, *d_pres, *d_sspd, *d_vol, *d_div, *d_mass, *d_force;
  const double* d_stress[2];  // reference bin rb, [9][ne]; null: the stress is zero
  const double* d_statev;     // [nsv][ne]
};

__global__ void __launch_bounds__(kBlock) k_down_elems(const ElemDown a) {
  __shared__ double buf[kBlock * 9];
  const int E0 = blockIdx.x * kBlock;
  const int E = E0 + threadIdx.x;
  const int cnt = min(kBlock, a.ne - E0);
  const int e = E < a.ne ? a.ext2int[E] : 0;
  if (E < a.ne) {
    if (a.statev)
      for (int k = 0; k < a.nsv; ++k) a.statev[(size_t)E * a.nsv + k] = a.d_statev[(size_t)k * a.ne + e];
    if (a.sie) {
      a.sie[E] = a.d_sie[0][e];
      a.sie[(size_t)a.ne + E] = a.d_sie[1][e];
    }
    if (a.den) a.den[E] = a.d_den[e];
    if (a.pres) a.pres[E] = a.d_pres[e];
    if (a.sspd) a.sspd[E] = a.d_sspd[e];
    if (a.vol) a.vol[E] = a.d_vol[e];
    if (a.div) a.div[E] = a.d_div[e];
    if (a.mass) a.mass[E] = a.d_mass[e];
  }
  if (a.stress) {
#pragma unroll
    for (int rb = 0; rb < 2; ++rb) {
      double* o = a.stress + ((size_t)rb * a.ne + E0) * 9;
      if (a.d_stress[rb]) {
        __syncthreads();
        if (E < a.ne)
#pragma unroll
          for (int k = 0; k < 9; ++k) buf[threadIdx.x * 9 + k] = a.d_stress[rb][(size_t)k * a.ne + e];
        __syncthreads();
        store_run(o, buf, cnt * 9);
      } else {
        for (int k = threadIdx.x; k < cnt * 9; k += kBlock) o[k] = 0.0;
      }
    }
  }
}

// Corner forces, device [lid*dims+dim][e] -> reference [(E*npe+lid)*dims+dim]
// (R = npe*dims = 24 or 8 values per element), 64 elements per block staged in
// shared memory.
constexpr int kForceChunk = 64;
__global__ void __launch_bounds__(kBlock) k_down_force(const ElemDown a) {
  __shared__ double buf[kForceChunk * 24];
  const int R = a.force_rows;
  const int E0 = blockIdx.x * kForceChunk;
  const int cnt = min(kForceChunk, a.ne - E0);
  for (int k = threadIdx.x; k < cnt * R; k += kBlock) {
    const int E = E0 + k / R, r = k % R;
    buf[k] = a.d_force[(size_t)r * a.ne + a.ext2int[E]];
  }
  __syncthreads();
  store_run(a.corner_force + (size_t)E0 * R, buf, cnt * R);
}

// Snapshot of the state for a graphics dump, in the caller's numbering, with
// the per-element fields write_outputs derives: the element speed from the
// average of its nodes' velocities (outputs.cpp:133-156) and the element
// centroid and radii of the state file (outputs.cpp:451-475), in the
// reference's operation order (this unit compiles without contraction).
__global__ void __launch_bounds__(kBlock) k_snap(const SnapArgs a) {
  if (!a.force && !a.ctrl->wrote) return;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t slot = (size_t)(*a.count % (unsigned long long)a.nslots);
  double* base = a.ring + slot * ((size_t)kSnapNodeRows * a.nn + (size_t)kSnapElemRows * a.ne);
  if (t < a.nn) {
    const int j = (int)t, i = a.node_ext2int[j];
    base[j] = a.x[i];
    base[(size_t)a.nn + j] = a.y[i];
    base[2 * (size_t)a.nn + j] = a.z[i];
    base[3 * (size_t)a.nn + j] = a.u[i];
    base[4 * (size_t)a.nn + j] = a.v[i];
    base[5 * (size_t)a.nn + j] = a.w[i];
  }
  if (t < a.ne) {
    const int E = (int)t, e = a.elem_ext2int[E];
    double* eb = base + (size_t)kSnapNodeRows * a.nn;
    const size_t ne = (size_t)a.ne;
    eb[E] = a.den[e];
    eb[ne + E] = a.pres[e];
    eb[2 * ne + E] = a.sie[e];
    eb[3 * ne + E] = a.vol[e];
    eb[4 * ne + E] = a.mass[e];
    eb[5 * ne + E] = a.sspd[e];
    double ev[3] = {0.0, 0.0, 0.0}, ec[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int l = 0; l < 8; ++l) {
      const int n = a.nie[(size_t)e * 8 + l];
      ev[0] += a.u[n];
      ev[1] += a.v[n];
      ev[2] += a.w[n];
      ec[0] += a.x[n];
      ec[1] += a.y[n];
      ec[2] += a.z[n];
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      ev[d] = ev[d] / 8.0;
      ec[d] = ec[d] / 8.0;
    }
    double speed_sqrd = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) speed_sqrd += ev[d] * ev[d];
    eb[6 * ne + E] = sqrt(speed_sqrd);
    eb[7 * ne + E] = (double)a.mat[e];
    eb[8 * ne + E] = ec[0];
    eb[9 * ne + E] = ec[1];
    eb[10 * ne + E] = ec[2];
    eb[11 * ne + E] = sqrt(ec[0] * ec[0] + ec[1] * ec[1]);
    eb[12 * ne + E] = sqrt(ec[0] * ec[0] + ec[1] * ec[1] + ec[2] * ec[2]);
  }
}

__global__ void k_snap_publish(const SnapArgs a) {
  if (!a.force && !a.ctrl->wrote) return;
  const unsigned long long c = *a.count;
  a.times[c % (unsigned long long)a.nslots] = a.ctrl->time_value;
  *a.count = c + 1;
  __threadfence_system();
  *(volatile unsigned long long*)a.produced = c + 1;
}

}  // namespace

void launch_snapshot(const SnapArgs& a, cudaStream_t s) {
  const long long n = a.nn > a.ne ? a.nn : a.ne;
  k_snap<<<blocks(n), kBlock, 0, s>>>(a);
  k_snap_publish<<<1, 1, 0, s>>>(a);
}

bool direct_host_access() {
  int dev = 0, v = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) return false;
  return v != 0;
}

int upload_state(fierro_sgh* h, const fierro_sgh_state* s, XferStatus* host_status, bool wait) {
  const int nn = (int)h->nn, ne = (int)h->ne;
  cudaStream_t stream = h->stream;
  XferStatus init{};
  init.flags = 0;
  for (int k = 0; k < XferStatus::COUNT; ++k) init.first[k] = LLONG_MAX;
  CUDA_TRY(cudaMemcpyAsync(h->d_xfer, &init, sizeof(init), cudaMemcpyHostToDevice, stream));
  const int D = h->dims == 2 ? 2 : 3;
  NodeUp nu{};
  nu.nn = nn;
  nu.dims = D;
  nu.ext2int = h->d_node_ext2int;
  nu.coords = s->node_coords;
  nu.vel = s->node_vel;
  nu.mass = s->node_mass;
  for (int b = 0; b < 2; ++b)
    for (int d = 0; d < D; ++d) {
      nu.x[b][d] = h->d_x[b][d];
      nu.v[b][d] = h->d_v[b][d];
    }
  nu.node_mass = h->d_node_mass;
  nu.st = h->d_xfer;
  k_up_nodes<<<blocks(nn), kBlock, 0, stream>>>(nu);
  ElemUp eu{};
  eu.ne = ne;
  eu.nmat = h->nmat;
  eu.nsv = (int)s->num_state_vars;
  eu.ext2int = h->d_elem_ext2int;
  eu.sie = s->elem_sie;
  eu.den = s->elem_den;
  eu.pres = s->elem_pres;
  eu.sspd = s->elem_sspd;
  eu.vol = s->elem_vol;
  eu.mass = s->elem_mass;
  eu.statev = s->elem_statev;
  eu.div = s->elem_div;
  eu.mat_id = s->elem_mat_id;
  eu.d_sie[0] = h->d_sie[0];
  eu.d_sie[1] = h->d_sie[1];
  eu.d_den = h->d_den;
  eu.d_pres = h->d_pres;
  eu.d_sspd = h->d_sspd;
  eu.d_vol = h->d_vol;
  eu.d_mass = h->d_elem_mass;
  eu.d_gamma = h->d_gamma;
  eu.d_csmin = h->d_csmin;
  eu.d_div = h->d_div[1];  // the caller's elem_div is what the reference shows before any stage runs
  eu.d_mat = h->d_mat;
  eu.st = h->d_xfer;
  if (h->strength) {
    eu.stress = s->elem_stress;
    eu.d_stress[0] = h->d_stress[0];
    eu.d_stress[1] = h->d_stress[1];
    eu.d_statev = h->d_statev;
    if (!s->elem_stress) {
      int dev = 0, sms = 0;
      CUDA_TRY(cudaGetDevice(&dev));
      CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
      for (int b = 0; b < 2; ++b) k_zero<<<sms * 4, kBlock, 0, stream>>>(h->d_stress[b], (long long)ne * 9);
    }
  }
  k_up_elems<<<blocks(ne), kBlock, 0, stream>>>(eu);
  if (s->elem_stress && !h->strength) {
    int dev = 0, sms = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    k_check_zero<<<sms * 8, kBlock, 0, stream>>>(s->elem_stress, (long long)ne * 18, h->d_xfer);
  }
  CUDA_TRY(cudaGetLastError());
  return wait ? finish_upload(h, host_status) : FIERRO_OK;
}

int finish_upload(fierro_sgh* h, XferStatus* host_status) {
  CUDA_TRY(cudaMemcpyAsync(host_status, h->d_xfer, sizeof(XferStatus), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  return FIERRO_OK;
}

int download_state(fierro_sgh* h, fierro_sgh_state* s, const int bins[2], int div_buffer, bool wait) {
  const int nn = (int)h->nn, ne = (int)h->ne;
  cudaStream_t stream = h->stream;
  const int D = h->dims == 2 ? 2 : 3;
  if (s->node_coords || s->node_vel || s->node_mass) {
    NodeDown nd{};
    nd.nn = nn;
    nd.dims = D;
    nd.ext2int = h->d_node_ext2int;
    nd.coords = s->node_coords;
    nd.vel = s->node_vel;
    nd.mass = s->node_mass;
    for (int rb = 0; rb < 2; ++rb)
      for (int d = 0; d < D; ++d) {
        nd.x[rb][d] = h->d_x[bins[rb]][d];
        nd.v[rb][d] = h->d_v[bins[rb]][d];
      }
    nd.node_mass = h->d_node_mass;
    k_down_nodes<<<blocks(nn), kBlock, 0, stream>>>(nd);
  }
  ElemDown ed{};
  ed.ne = ne;
  ed.force_rows = D == 2 ? 8 : 24;
  ed.ext2int = h->d_elem_ext2int;
  ed.sie = s->elem_sie;
  ed.den = s->elem_den;
  ed.pres = s->elem_pres;
  ed.sspd = s->elem_sspd;
  ed.vol = s->elem_vol;
  ed.div = s->elem_div;
  ed.mass = s->elem_mass;
  ed.stress = s->elem_stress;
  ed.corner_force = s->corner_force;
  ed.d_sie[0] = h->d_sie[bins[0]];
  ed.d_sie[1] = h->d_sie[bins[1]];
  ed.d_den = h->d_den;
  ed.d_pres = h->d_pres;
  ed.d_sspd = h->d_sspd;
  ed.d_vol = h->d_vol;
  ed.d_div = h->d_div[div_buffer];
  ed.d_mass = h->d_elem_mass;
  ed.d_force = h->d_force;
  if (h->strength) {
    ed.d_stress[0] = h->d_stress[bins[0]];
    ed.d_stress[1] = h->d_stress[bins[1]];
    ed.statev = s->elem_statev;
    ed.nsv = (int)h->nsv;
    ed.d_statev = h->d_statev;
  }
  k_down_elems<<<blocks(ne), kBlock, 0, stream>>>(ed);
  if (s->corner_force) k_down_force<<<(unsigned)((ne + kForceChunk - 1) / kForceChunk), kBlock, 0, stream>>>(ed);
  CUDA_TRY(cudaGetLastError());
  if (wait) CUDA_TRY(cudaStreamSynchronize(stream));
  return FIERRO_OK;
}

}  // namespace xfer
}  // namespace fierro
