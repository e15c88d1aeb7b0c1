// The initial state on the GPU: setup (setup.cpp:10-424) after get_vol
// (driver.cpp:239), in the caller's numbering, for fierro_sgh_setup.  The same
// operations in the same order as the host set-up (sgh_host.cpp), compiled
// without contraction, so the two give the same doubles:
//   element volumes (geometry.cpp:271-310, generated straight-line code),
//   boundary patches and node masks (mesh.h:501-515, setup.cpp:431-665),
//   fills in deck order (setup.cpp:109-357: region test on the element centroid,
//   density, mass, energy, state variables, ideal-gas EOS, node velocities),
//   boundary velocities (setup.cpp:362), node masses summed over each node's
//   elements in ascending element id (setup.cpp:394-420).
// The tg_vortex velocity fill needs libm's sin / cos and stays on the host.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "sgh_handle.h"
#include "sgh_hex.h"
#include "sgh_setup.h"

#define FIERRO_FMA 0

namespace fierro {
namespace setup_gpu {
namespace {

#include "sgh_sort.cuh"
#include "sgh_hex_geometry.cuh"

constexpr int kBlock = 256;
unsigned nblk(long long n) { return (unsigned)((n + kBlock - 1) / kBlock); }

struct Status {
  enum { NODE_ID = 0, REPEAT = 1, COORD = 2, VOLUME = 3, COUNT = 4 };
  unsigned flags;
  int pad;
  long long first[COUNT];
};

__device__ __forceinline__ void flag(Status* st, int which, long long idx) {
  atomicOr(&st->flags, 1u << which);
  atomicMin(&st->first[which], idx);
}

__global__ void k_read(int ne, int nn, const uint64_t* __restrict__ nie_h, const double* __restrict__ xyz_h,
                       int* __restrict__ nie, double* __restrict__ xyz, Status* st) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < ne) {
    const int E = (int)t;
    uint64_t n[8];
#pragma unroll
    for (int l = 0; l < 8; ++l) n[l] = nie_h[(size_t)E * 8 + l];
#pragma unroll
    for (int l = 0; l < 8; ++l) {
      if (n[l] >= (uint64_t)nn) flag(st, Status::NODE_ID, E);
      for (int k = 0; k < l; ++k)
        if (n[k] == n[l]) flag(st, Status::REPEAT, E);
      nie[(size_t)E * 8 + l] = n[l] < (uint64_t)nn ? (int)n[l] : 0;
    }
  }
  if (t < (long long)nn * 3) {
    const double v = xyz_h[t];
    xyz[t] = v;
    if (!isfinite(v)) flag(st, Status::COORD, t);
  }
}

__global__ void k_volume(int ne, const int* __restrict__ nie, const double* __restrict__ xyz,
                         double* __restrict__ vol, Status* st) {
  const int E = blockIdx.x * blockDim.x + threadIdx.x;
  if (E >= ne) return;
  double x[8], y[8], z[8];
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    const double* c = xyz + (size_t)nie[(size_t)E * 8 + l] * 3;
    x[l] = c[0];
    y[l] = c[1];
    z[l] = c[2];
  }
  const double v = hex_volume(x, y, z);
  vol[E] = v;
  if (!(v > 0.0) || !isfinite(v)) flag(st, Status::VOLUME, E);
}

// Corners in caller order, keyed by node: a stable sort lists each node's
// elements in ascending id (the corner order of mesh.h:218-241).
__global__ void k_corners(int ne, const int* __restrict__ nie, uint64_t* __restrict__ key, int* __restrict__ val,
                          unsigned* __restrict__ cnt) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (long long)ne * 8) return;
  const int n = nie[k];
  key[k] = (uint64_t)n;
  val[k] = (int)(k >> 3);
  atomicAdd(&cnt[n], 1u);
}

constexpr unsigned long long pack_faces(int f0) {
  unsigned long long w = 0;
  for (int f = 0; f < 3; ++f)
    for (int k = 0; k < 4; ++k) w |= (unsigned long long)hex::PATCH[f0 + f][k] << (3 * (f * 4 + k));
  return w;
}
constexpr unsigned long long kFaces0 = pack_faces(0), kFaces1 = pack_faces(3);
__device__ __forceinline__ int face_lid(int f, int k) {
  return (int)(((f < 3 ? kFaces0 : kFaces1) >> (3 * ((f % 3) * 4 + k))) & 7);
}

struct Bc {
  int surface, bits;
  double value;
};

__device__ __forceinline__ bool on_surface(const double* c, int tag, double val) {
  if (tag == 0) return fabs(c[0] - val) <= 1.0e-7;
  if (tag == 1) return fabs(c[1] - val) <= 1.0e-7;
  if (tag == 2) return fabs(c[2] - val) <= 1.0e-7;
  if (tag == 3) return fabs(sqrt(c[0] * c[0] + c[1] * c[1]) - val) <= 1.0e-7;
  if (tag == 4) return fabs(sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]) - val) <= 1.0e-7;
  return false;
}

__device__ __forceinline__ bool elem_has(const int* nie, int o, int n) {
#pragma unroll
  for (int l = 0; l < 8; ++l)
    if (nie[(size_t)o * 8 + l] == n) return true;
  return false;
}

__global__ void k_patches(int ne, const int* __restrict__ nie, const unsigned* __restrict__ start,
                          const int* __restrict__ elems, const double* __restrict__ xyz, const Bc* __restrict__ bcs,
                          int nbcs, unsigned* __restrict__ mask) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ne * 6) return;
  const int E = (int)(t / 6), f = (int)(t % 6);
  int fn[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) fn[k] = nie[(size_t)E * 8 + face_lid(f, k)];
  for (unsigned c = start[fn[0]]; c < start[fn[0] + 1]; ++c) {
    const int o = elems[c];
    if (o != E && elem_has(nie, o, fn[1]) && elem_has(nie, o, fn[2]) && elem_has(nie, o, fn[3])) return;
  }
  for (int s = 0; s < nbcs; ++s) {
    bool all = true;
    for (int k = 0; k < 4 && all; ++k) all = on_surface(xyz + (size_t)fn[k] * 3, bcs[s].surface, bcs[s].value);
    if (all)
      for (int k = 0; k < 4; ++k) atomicOr(&mask[fn[k]], (unsigned)bcs[s].bits);
  }
}

struct Fill {
  int volume, mat_id, velocity;
  double x1, x2, y1, y2, z1, z2, radius1, radius2, u, v, w, speed, sie, den;
};

struct ElemOut {
  double *den, *mass, *sie, *pres, *sspd, *statev;
  uint64_t* mat;
  double* vel;  // [nn][3], bin 1
};

__global__ void k_fill(int ne, int nsv, const Fill F, const int* __restrict__ nie, const double* __restrict__ xyz,
                       const double* __restrict__ vol, const double* __restrict__ state_vars, ElemOut o) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  double ec[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    const double* c = xyz + (size_t)nie[(size_t)e * 8 + l] * 3;
    ec[0] += c[0];
    ec[1] += c[1];
    ec[2] += c[2];
  }
  ec[0] = ec[0] / 8;
  ec[1] = ec[1] / 8;
  ec[2] = ec[2] / 8;
  const double radius = sqrt(ec[0] * ec[0] + ec[1] * ec[1] + ec[2] * ec[2]);
  const double radius_cyl = sqrt(ec[0] * ec[0] + ec[1] * ec[1]);
  bool fill_this = false;
  switch (F.volume) {
    case 0: fill_this = true; break;
    case 1:
      fill_this = ec[0] >= F.x1 && ec[0] <= F.x2 && ec[1] >= F.y1 && ec[1] <= F.y2 && ec[2] >= F.z1 && ec[2] <= F.z2;
      break;
    case 2: fill_this = radius_cyl >= F.radius1 && radius_cyl <= F.radius2; break;
    case 3: fill_this = radius >= F.radius1 && radius <= F.radius2; break;
  }
  if (!fill_this) return;
  double* sv = o.statev + (size_t)e * nsv;
  o.den[e] = F.den;
  o.mass[e] = o.den[e] * vol[e];
  o.sie[e] = F.sie;
  o.mat[e] = (uint64_t)F.mat_id;
  for (int v = 0; v < nsv; ++v) sv[v] = state_vars[(size_t)F.mat_id * nsv + v];
  // ideal_gas (eos.cpp:12-46)
  const double gamma = sv[0], csmin = sv[1];
  o.pres[e] = (gamma - 1.0) * o.sie[e] * o.den[e];
  double c = sqrt(gamma * (gamma - 1.0) * o.sie[e]);
  if (c < csmin) c = csmin;
  o.sspd[e] = c;
  for (int l = 0; l < 8; ++l) {
    const int n = nie[(size_t)e * 8 + l];
    const double* x = xyz + (size_t)n * 3;
    double* v = o.vel + (size_t)n * 3;
    if (F.velocity == 0) {
      v[0] = F.u;
      v[1] = F.v;
      v[2] = F.w;
    } else if (F.velocity == 1 || F.velocity == 2) {
      const int nd = (F.velocity == 1) ? 2 : 3;
      double dir[3] = {0.0, 0.0, 0.0};
      double radius_val = 0.0;
      for (int d = 0; d < nd; ++d) {
        dir[d] = x[d];
        radius_val += x[d] * x[d];
      }
      radius_val = sqrt(radius_val);
      for (int d = 0; d < nd; ++d) {
        if (radius_val > 1.0e-14) dir[d] /= (radius_val);
        else dir[d] = 0.0;
      }
      v[0] = F.speed * dir[0];
      v[1] = F.speed * dir[1];
      v[2] = (nd == 3) ? F.speed * dir[2] : 0.0;
    }
  }
}

__global__ void k_nodes(int nn, const unsigned* __restrict__ mask, const unsigned* __restrict__ start,
                        const int* __restrict__ elems, const double* __restrict__ mass, double* __restrict__ vel,
                        double* __restrict__ node_mass) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  const unsigned m = mask[n];
#pragma unroll
  for (int d = 0; d < 3; ++d)
    if (m & (1u << d)) vel[(size_t)n * 3 + d] = 0.0;
  double s = 0.0;
  for (unsigned k = start[n]; k < start[n + 1]; ++k) s += 1.0 / 8.0 * mass[elems[k]];
  node_mass[n] = s;
}

// Host memset in parallel (also makes the pages resident).
void zero(void* p, size_t bytes) {
  if (!p || !bytes) return;
  char* c = static_cast<char*>(p);
  const int64_t chunk = 1 << 22;
  const int64_t n = (int64_t)((bytes + chunk - 1) / chunk);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    const size_t off = (size_t)i * chunk;
    std::memset(c + off, 0, std::min<size_t>(chunk, bytes - off));
  }
}

}  // namespace

bool usable(const fierro_mat_fill* fills, int64_t num_fills) {
  if (!xfer::direct_host_access()) return false;
  for (int64_t f = 0; f < num_fills; ++f)
    if (fills[f].velocity == 5) return false;  // tg_vortex: libm sin / cos on the host
  return true;
}

int run(const fierro_mesh* mesh, const double* state_vars, int64_t num_state_vars, const fierro_mat_fill* fills,
        int64_t num_fills, const fierro_boundary* boundaries, int64_t num_bcs, fierro_sgh_state* out) {
  const int nn = (int)mesh->num_nodes, ne = (int)mesh->num_elems, nsv = (int)num_state_vars;
  cudaStream_t st = nullptr;
  CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
  } guard{st};
  Scratch sc;
  int* nie = nullptr;
  double *xyz = nullptr, *vol = nullptr;
  Status* d_st = nullptr;
  TRY(sc.alloc(&nie, (size_t)ne * 8));
  TRY(sc.alloc(&xyz, (size_t)nn * 3));
  TRY(sc.alloc(&vol, (size_t)ne));
  TRY(sc.alloc(&d_st, 1));
  Status hs{};
  for (int k = 0; k < Status::COUNT; ++k) hs.first[k] = LLONG_MAX;
  CUDA_TRY(cudaMemcpyAsync(d_st, &hs, sizeof(hs), cudaMemcpyHostToDevice, st));
  k_read<<<nblk(std::max<long long>(ne, (long long)nn * 3)), kBlock, 0, st>>>(ne, nn, mesh->nodes_in_elem,
                                                                              mesh->coords, nie, xyz, d_st);
  k_volume<<<nblk(ne), kBlock, 0, st>>>(ne, nie, xyz, vol, d_st);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(&hs, d_st, sizeof(hs), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (hs.flags & (1u << Status::NODE_ID))
    return set_error(FIERRO_EINVAL, "element %lld has a node id out of range", hs.first[Status::NODE_ID]);
  if (hs.flags & (1u << Status::REPEAT))
    return set_error(FIERRO_EINVAL, "element %lld repeats a node", hs.first[Status::REPEAT]);
  if (hs.flags & (1u << Status::COORD))
    return set_error(FIERRO_EINVAL, "non-finite coordinate at %lld", hs.first[Status::COORD]);
  if (hs.flags & (1u << Status::VOLUME))
    return set_error(FIERRO_ENUMERIC, "setup: element %lld has a non-positive volume (inverted or degenerate)",
                     hs.first[Status::VOLUME]);
  // node -> elements, ascending element id
  const long long nc = (long long)ne * 8;
  uint64_t *ck = nullptr, *ck2 = nullptr;
  int *cv = nullptr, *cv2 = nullptr;
  unsigned *cnt = nullptr, *start = nullptr;
  TRY(sc.alloc(&ck, (size_t)nc));
  TRY(sc.alloc(&ck2, (size_t)nc));
  TRY(sc.alloc(&cv, (size_t)nc));
  TRY(sc.alloc(&cv2, (size_t)nc));
  TRY(sc.alloc(&cnt, (size_t)nn + 1));
  TRY(sc.alloc(&start, (size_t)nn + 1));
  CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(unsigned) * (nn + 1), st));
  k_corners<<<nblk(nc), kBlock, 0, st>>>(ne, nie, ck, cv, cnt);
  int bits = 1;
  while ((1LL << bits) < (long long)nn) ++bits;
  uint64_t* k = ck;
  int* elems = cv;
  TRY(radix_sort(sc, &k, &elems, ck2, cv2, (int)nc, bits, st));
  TRY(exclusive_scan(sc, cnt, start, (long long)nn + 1, st));
  // boundary masks
  std::vector<Bc> hb((size_t)num_bcs);
  for (int64_t s = 0; s < num_bcs; ++s)
    hb[s] = {boundaries[s].surface, (int)bc_mask_bits(boundaries[s].hydro_bc, boundaries[s].surface, 3),
             boundaries[s].value};
  Bc* d_bcs = nullptr;
  unsigned* mask = nullptr;
  TRY(sc.alloc(&d_bcs, hb.size()));
  TRY(sc.alloc(&mask, (size_t)nn));
  if (!hb.empty()) CUDA_TRY(cudaMemcpyAsync(d_bcs, hb.data(), sizeof(Bc) * hb.size(), cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemsetAsync(mask, 0, sizeof(unsigned) * nn, st));
  k_patches<<<nblk(nc / 8 * 6), kBlock, 0, st>>>(ne, nie, start, elems, xyz, d_bcs, (int)num_bcs, mask);
  // fills, in deck order
  ElemOut eo{};
  double *den = nullptr, *mass = nullptr, *sie = nullptr, *pres = nullptr, *sspd = nullptr, *statev = nullptr,
         *vel = nullptr, *nmass = nullptr;
  uint64_t* mat = nullptr;
  TRY(sc.alloc(&den, (size_t)ne));
  TRY(sc.alloc(&mass, (size_t)ne));
  TRY(sc.alloc(&sie, (size_t)ne));
  TRY(sc.alloc(&pres, (size_t)ne));
  TRY(sc.alloc(&sspd, (size_t)ne));
  TRY(sc.alloc(&statev, (size_t)ne * nsv));
  TRY(sc.alloc(&mat, (size_t)ne));
  TRY(sc.alloc(&vel, (size_t)nn * 3));
  TRY(sc.alloc(&nmass, (size_t)nn));
  double* zero_targets[] = {den, mass, sie, pres, sspd};
  for (double* p : zero_targets) CUDA_TRY(cudaMemsetAsync(p, 0, sizeof(double) * ne, st));
  CUDA_TRY(cudaMemsetAsync(statev, 0, sizeof(double) * ne * nsv, st));
  CUDA_TRY(cudaMemsetAsync(mat, 0, sizeof(uint64_t) * ne, st));
  CUDA_TRY(cudaMemsetAsync(vel, 0, sizeof(double) * nn * 3, st));
  int64_t nmat_used = 0;
  for (int64_t f = 0; f < num_fills; ++f) nmat_used = std::max<int64_t>(nmat_used, fills[f].mat_id + 1);
  double* d_svars = nullptr;
  TRY(sc.alloc(&d_svars, (size_t)std::max<int64_t>(nmat_used, 1) * nsv));
  if (nmat_used > 0)
    CUDA_TRY(cudaMemcpyAsync(d_svars, state_vars, sizeof(double) * nmat_used * nsv, cudaMemcpyHostToDevice, st));
  eo.den = den;
  eo.mass = mass;
  eo.sie = sie;
  eo.pres = pres;
  eo.sspd = sspd;
  eo.statev = statev;
  eo.mat = mat;
  eo.vel = vel;
  for (int64_t f = 0; f < num_fills; ++f) {
    const fierro_mat_fill& F = fills[f];
    Fill d{F.volume, F.mat_id, F.velocity, F.x1, F.x2, F.y1, F.y2, F.z1, F.z2, F.radius1, F.radius2,
           F.u, F.v, F.w, F.speed, F.sie, F.den};
    k_fill<<<nblk(ne), kBlock, 0, st>>>(ne, nsv, d, nie, xyz, vol, d_svars, eo);
  }
  k_nodes<<<nblk(nn), kBlock, 0, st>>>(nn, mask, start, elems, mass, vel, nmass);
  CUDA_TRY(cudaGetLastError());
  // results into the caller's arrays (caller numbering: plain copies)
  const size_t bn = sizeof(double) * (size_t)nn, be = sizeof(double) * (size_t)ne;
  zero(out->node_vel, bn * 3);             // bin 0
  zero(out->elem_sie, be);                 // bin 0
  zero(out->elem_stress, be * 18);
  zero(out->elem_div, be);
  zero(out->corner_force, be * 24);
  CUDA_TRY(cudaMemcpyAsync(out->node_coords, xyz, bn * 3, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(out->node_coords + (size_t)nn * 3, xyz, bn * 3, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(out->node_vel + (size_t)nn * 3, vel, bn * 3, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(out->node_mass, nmass, bn, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(out->elem_den, den, be, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(out->elem_pres, pres, be, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(out->elem_sspd, sspd, be, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(out->elem_sie + ne, sie, be, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(out->elem_vol, vol, be, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(out->elem_mass, mass, be, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(out->elem_mat_id, mat, sizeof(uint64_t) * ne, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(out->elem_statev, statev, be * nsv, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  return FIERRO_OK;
}

}  // namespace setup_gpu
}  // namespace fierro
