// Mesh topology on the GPU: validation, Morton renumbering, corner and
// neighbour CSR and boundary node masks (the work of mesh.h:180-649 and
// setup.cpp:431-665), built from the caller's host arrays by kernels that read
// them in place.  Integer work only, apart from the Morton quantisation and the
// boundary-surface test, whose floating-point operations are those of the host
// builder (compiled without contraction), so the result is the same topology:
//   * elements and nodes ordered by 63-bit Morton keys of centroid / position,
//     ties by caller id (stable LSD radix sort, 8-bit digits);
//   * each node's corners in ascending caller element id (the summation order of
//     update_velocity_sgh, mesh.h:218-241): a stable sort of the corners, listed
//     in caller order, by internal node id;
//   * each element's neighbours in the order its local nodes and their corner
//     lists meet them, without repeats;
//   * a face is a boundary patch when no other element holds its four nodes
//     (mesh.h:501-515); a boundary set takes the nodes of the patches whose four
//     nodes lie on its surface (check_bdy, setup.cpp:487-571).
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <vector>

#include "sgh_handle.h"
#include "sgh_hex.h"
#include "sgh_topo.h"

namespace fierro {
namespace topo {
namespace {
#include "sgh_sort.cuh"
}  // namespace
}  // namespace topo
}  // namespace fierro

namespace fierro {
namespace topo {
namespace {

constexpr int kBlock = 256;

unsigned nblk(long long n, int b = kBlock) { return (unsigned)((n + b - 1) / b); }

// ---------------------------------------------------------------- validation
struct MeshStatus {
  unsigned flags;  // 1: node id out of range, 2: repeated node, 4: non-finite coordinate
  int pad;
  long long first[3];
};

__device__ __forceinline__ void flag(MeshStatus* st, int which, long long idx) {
  atomicOr(&st->flags, 1u << which);
  atomicMin(&st->first[which], idx);
}

__global__ void k_read_elems(int ne, int nn, const uint64_t* __restrict__ nie, int* __restrict__ out,
                             MeshStatus* st) {
  const int E = blockIdx.x * blockDim.x + threadIdx.x;
  if (E >= ne) return;
  uint64_t n[8];
#pragma unroll
  for (int l = 0; l < 8; ++l) n[l] = nie[(size_t)E * 8 + l];
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    if (n[l] >= (uint64_t)nn) flag(st, 0, E);
    for (int k = 0; k < l; ++k)
      if (n[k] == n[l]) flag(st, 1, E);
    out[(size_t)E * 8 + l] = n[l] < (uint64_t)nn ? (int)n[l] : 0;
  }
}

__device__ __forceinline__ long long okey(double d) {
  const long long b = __double_as_longlong(d);
  return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL);
}
__device__ __forceinline__ double okey_decode(long long k) {
  return __longlong_as_double(k ^ ((k >> 63) & 0x7FFFFFFFFFFFFFFFLL));
}

// Coordinates (copied to the device) and their bounding box, as order keys.
__global__ void k_read_nodes(int nn, const double* __restrict__ c, double* __restrict__ out, long long* box,
                             MeshStatus* st) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  long long lo[3] = {LLONG_MAX, LLONG_MAX, LLONG_MAX}, hi[3] = {LLONG_MIN, LLONG_MIN, LLONG_MIN};
  if (j < nn) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double v = c[(size_t)j * 3 + d];
      out[(size_t)j * 3 + d] = v;
      if (!isfinite(v)) flag(st, 2, (long long)j * 3 + d);
      lo[d] = okey(v);
      hi[d] = okey(v);
    }
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[d] = min(lo[d], __shfl_xor_sync(0xFFFFFFFFu, lo[d], o));
      hi[d] = max(hi[d], __shfl_xor_sync(0xFFFFFFFFu, hi[d], o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&box[d], lo[d]);
      atomicMax(&box[3 + d], hi[d]);
    }
  }
}

// Element centroids (the host builder's operation order) and their bounding box.
__global__ void k_centroids(int ne, const int* __restrict__ nie, const double* __restrict__ xyz,
                            double* __restrict__ cen, long long* box) {
  const int E = blockIdx.x * blockDim.x + threadIdx.x;
  long long lo[3] = {LLONG_MAX, LLONG_MAX, LLONG_MAX}, hi[3] = {LLONG_MIN, LLONG_MIN, LLONG_MIN};
  if (E < ne) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      double s = 0;
#pragma unroll
      for (int l = 0; l < 8; ++l) s += xyz[(size_t)nie[(size_t)E * 8 + l] * 3 + d];
      const double v = s * 0.125;
      cen[(size_t)E * 3 + d] = v;
      lo[d] = okey(v);
      hi[d] = okey(v);
    }
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[d] = min(lo[d], __shfl_xor_sync(0xFFFFFFFFu, lo[d], o));
      hi[d] = max(hi[d], __shfl_xor_sync(0xFFFFFFFFu, hi[d], o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&box[d], lo[d]);
      atomicMax(&box[3 + d], hi[d]);
    }
  }
}

__device__ __forceinline__ uint64_t spread21(uint64_t v) {
  v &= 0x1FFFFF;
  v = (v | (v << 32)) & 0x1F00000000FFFFULL;
  v = (v | (v << 16)) & 0x1F0000FF0000FFULL;
  v = (v | (v << 8)) & 0x100F00F00F00F00FULL;
  v = (v | (v << 4)) & 0x10C30C30C30C30C3ULL;
  v = (v | (v << 2)) & 0x1249249249249249ULL;
  return v;
}

// Morton keys quantised on the bounding box to 21 bits per axis (the host
// builder's arithmetic), with the identity as the sort's values.
__global__ void k_morton(int n, const double* __restrict__ pts, const long long* __restrict__ box,
                         uint64_t* __restrict__ key, int* __restrict__ val) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t q[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double lo = okey_decode(box[d]), hi = okey_decode(box[3 + d]);
    const double span = hi - lo;
    const double f = span > 0 ? (pts[(size_t)i * 3 + d] - lo) / span : 0.0;
    q[d] = (uint64_t)fmin(2097151.0, fmax(0.0, f * 2097151.0));
  }
  key[i] = spread21(q[0]) | (spread21(q[1]) << 1) | (spread21(q[2]) << 2);
  val[i] = i;
}

// ---------------------------------------------------------------- topology kernels
__global__ void k_invert(int n, const int* __restrict__ int2ext, int* __restrict__ ext2int) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) ext2int[int2ext[i]] = i;
}

__global__ void k_nie_internal(int ne, const int* __restrict__ nie_ext, const int* __restrict__ elem_int2ext,
                               const int* __restrict__ node_ext2int, int* __restrict__ nie) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int E = elem_int2ext[e];
#pragma unroll
  for (int l = 0; l < 8; ++l) nie[(size_t)e * 8 + l] = node_ext2int[nie_ext[(size_t)E * 8 + l]];
}

// Corners listed in caller order (E ascending, then lid): key = internal node,
// value = internal corner id; the per-node counts for the CSR.
__global__ void k_corner_keys(int ne, const int* __restrict__ nie_ext, const int* __restrict__ node_ext2int,
                              const int* __restrict__ elem_ext2int, uint64_t* __restrict__ key,
                              int* __restrict__ val, unsigned* __restrict__ node_count) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (long long)ne * 8) return;
  const int E = (int)(k >> 3), l = (int)(k & 7);
  const int n = node_ext2int[nie_ext[k]];
  key[k] = (uint64_t)n;
  val[k] = elem_ext2int[E] * 8 + l;
  atomicAdd(&node_count[n], 1u);
}

__global__ void k_to_int(long long n, const unsigned* __restrict__ in, int* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (int)in[i];
}

constexpr int kMaxNb = 64;  // distinct neighbours per element (26 in a conforming hex mesh)

// Neighbours of internal element e in the host builder's order (its local nodes
// in order, each node's corners in CSR order, repeats and e itself skipped);
// out (may be null) receives them.  Returns the count, or -1 beyond kMaxNb.
__device__ int neighbours(int e, const int* __restrict__ nie, const int* __restrict__ cin_start,
                          const int* __restrict__ cin, int* out) {
  int buf[kMaxNb];
  int k = 0;
  for (int l = 0; l < 8; ++l) {
    const int n = nie[(size_t)e * 8 + l];
    for (int c = cin_start[n]; c < cin_start[n + 1]; ++c) {
      const int o = cin[c] >> 3;
      if (o == e) continue;
      bool seen = false;
      for (int i = 0; i < k; ++i)
        if (buf[i] == o) {
          seen = true;
          break;
        }
      if (seen) continue;
      if (k == kMaxNb) return -1;
      buf[k] = o;
      if (out) out[k] = o;
      ++k;
    }
  }
  return k;
}

__global__ void k_nb_count(int ne, const int* __restrict__ nie, const int* __restrict__ cin_start,
                           const int* __restrict__ cin, unsigned* __restrict__ cnt, int* overflow) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int k = neighbours(e, nie, cin_start, cin, nullptr);
  if (k < 0) atomicOr(overflow, 1);
  cnt[e] = k < 0 ? 0u : (unsigned)k;
}

__global__ void k_nb_fill(int ne, const int* __restrict__ nie, const int* __restrict__ cin_start,
                          const int* __restrict__ cin, const int* __restrict__ eie_start, int* __restrict__ eie) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  neighbours(e, nie, cin_start, cin, eie + eie_start[e]);
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

// Face lids of hex::PATCH packed 3 bits each (faces 0-2 in the first word, 3-5
// in the second) so device code reads them as compile-time scalars.
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

__device__ __forceinline__ bool elem_has(const int* nie, int o, int n) {
#pragma unroll
  for (int l = 0; l < 8; ++l)
    if (nie[(size_t)o * 8 + l] == n) return true;
  return false;
}

// One thread per (element, face): boundary patch test, then the node masks of
// every boundary set whose surface holds the patch.
__global__ void k_patches(int ne, const int* __restrict__ nie, const int* __restrict__ cin_start,
                          const int* __restrict__ cin, const double* __restrict__ xyz_ext,
                          const int* __restrict__ node_int2ext, const Bc* __restrict__ bcs, int nbcs,
                          unsigned* __restrict__ mask) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ne * 6) return;
  const int e = (int)(t / 6), f = (int)(t % 6);
  int fn[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) fn[k] = nie[(size_t)e * 8 + face_lid(f, k)];
  for (int c = cin_start[fn[0]]; c < cin_start[fn[0] + 1]; ++c) {
    const int o = cin[c] >> 3;
    if (o != e && elem_has(nie, o, fn[1]) && elem_has(nie, o, fn[2]) && elem_has(nie, o, fn[3])) return;
  }
  for (int s = 0; s < nbcs; ++s) {
    bool all = true;
    for (int k = 0; k < 4 && all; ++k)
      all = on_surface(xyz_ext + (size_t)node_int2ext[fn[k]] * 3, bcs[s].surface, bcs[s].value);
    if (all)
      for (int k = 0; k < 4; ++k) atomicOr(&mask[fn[k]], (unsigned)bcs[s].bits);
  }
}

__global__ void k_mask_u8(int nn, const unsigned* __restrict__ in, unsigned char* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nn) out[i] = (unsigned char)in[i];
}

}  // namespace

int build_device(fierro_sgh* h, const fierro_mesh* mesh, const fierro_boundary* bcs, int64_t num_bcs) {
  const int nn = (int)mesh->num_nodes, ne = (int)mesh->num_elems;
  cudaStream_t st = h->stream;
  Scratch sc;
  // ---- caller arrays, read by the GPU; validation
  int* nie_ext = nullptr;
  double* xyz = nullptr;
  MeshStatus* d_ms = nullptr;
  long long* box = nullptr;  // [0..6) nodes, [6..12) centroids
  TRY(sc.alloc(&nie_ext, (size_t)ne * 8));
  TRY(sc.alloc(&xyz, (size_t)nn * 3));
  TRY(sc.alloc(&d_ms, 1));
  TRY(sc.alloc(&box, 12));
  MeshStatus ms{};
  ms.first[0] = ms.first[1] = ms.first[2] = LLONG_MAX;
  long long box0[12];
  for (int i = 0; i < 12; ++i) box0[i] = (i % 6) < 3 ? LLONG_MAX : LLONG_MIN;
  CUDA_TRY(cudaMemcpyAsync(d_ms, &ms, sizeof(ms), cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(box, box0, sizeof(box0), cudaMemcpyHostToDevice, st));
  k_read_elems<<<nblk(ne), kBlock, 0, st>>>(ne, nn, mesh->nodes_in_elem, nie_ext, d_ms);
  k_read_nodes<<<nblk(nn), kBlock, 0, st>>>(nn, mesh->coords, xyz, box, d_ms);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(&ms, d_ms, sizeof(ms), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (ms.flags & 1u) return set_error(FIERRO_EINVAL, "element %lld has a node id out of range", ms.first[0]);
  if (ms.flags & 2u) return set_error(FIERRO_EINVAL, "element %lld repeats a node", ms.first[1]);
  if (ms.flags & 4u) return set_error(FIERRO_EINVAL, "non-finite coordinate at %lld", ms.first[2]);
  // ---- Morton renumbering
  double* cen = nullptr;
  uint64_t *ka = nullptr, *kb = nullptr;
  int *va = nullptr, *vb = nullptr;
  const int nmax = std::max(nn, ne);
  TRY(sc.alloc(&cen, (size_t)ne * 3));
  TRY(sc.alloc(&ka, (size_t)nmax));
  TRY(sc.alloc(&kb, (size_t)nmax));
  TRY(sc.alloc(&va, (size_t)nmax));
  TRY(sc.alloc(&vb, (size_t)nmax));
  k_centroids<<<nblk(ne), kBlock, 0, st>>>(ne, nie_ext, xyz, cen, box + 6);
  int* elem_int2ext = h->d_elem_int2ext;
  int* node_int2ext = h->d_node_int2ext;
  {
    uint64_t* k = ka;
    int* v = va;
    k_morton<<<nblk(ne), kBlock, 0, st>>>(ne, cen, box + 6, k, v);
    TRY(radix_sort(sc, &k, &v, kb, vb, ne, 63, st));
    CUDA_TRY(cudaMemcpyAsync(elem_int2ext, v, sizeof(int) * ne, cudaMemcpyDeviceToDevice, st));
    k = ka;
    v = va;
    k_morton<<<nblk(nn), kBlock, 0, st>>>(nn, xyz, box, k, v);
    TRY(radix_sort(sc, &k, &v, kb, vb, nn, 63, st));
    CUDA_TRY(cudaMemcpyAsync(node_int2ext, v, sizeof(int) * nn, cudaMemcpyDeviceToDevice, st));
  }
  k_invert<<<nblk(ne), kBlock, 0, st>>>(ne, elem_int2ext, h->d_elem_ext2int);
  k_invert<<<nblk(nn), kBlock, 0, st>>>(nn, node_int2ext, h->d_node_ext2int);
  k_nie_internal<<<nblk(ne), kBlock, 0, st>>>(ne, nie_ext, elem_int2ext, h->d_node_ext2int, h->d_nie);
  // ---- corner CSR: corners in caller order, stably sorted by internal node
  const long long nc = (long long)ne * 8;
  uint64_t *ck = nullptr, *ck2 = nullptr;
  int *cv = nullptr, *cv2 = nullptr;
  unsigned *ncount = nullptr, *nstart = nullptr;
  TRY(sc.alloc(&ck, (size_t)nc));
  TRY(sc.alloc(&ck2, (size_t)nc));
  TRY(sc.alloc(&cv, (size_t)nc));
  TRY(sc.alloc(&cv2, (size_t)nc));
  TRY(sc.alloc(&ncount, (size_t)nn + 1));
  TRY(sc.alloc(&nstart, (size_t)nn + 1));
  CUDA_TRY(cudaMemsetAsync(ncount, 0, sizeof(unsigned) * (nn + 1), st));
  k_corner_keys<<<nblk(nc), kBlock, 0, st>>>(ne, nie_ext, h->d_node_ext2int, h->d_elem_ext2int, ck, cv, ncount);
  {
    int bits = 1;
    while ((1LL << bits) < (long long)nn) ++bits;
    uint64_t* k = ck;
    int* v = cv;
    TRY(radix_sort(sc, &k, &v, ck2, cv2, (int)nc, bits, st));
    CUDA_TRY(cudaMemcpyAsync(h->d_cin, v, sizeof(int) * nc, cudaMemcpyDeviceToDevice, st));
  }
  TRY(exclusive_scan(sc, ncount, nstart, (long long)nn + 1, st));
  k_to_int<<<nblk(nn + 1), kBlock, 0, st>>>(nn + 1, nstart, h->d_cin_start);
  // ---- neighbour CSR
  unsigned *nbc = nullptr, *nbs = nullptr;
  int* d_over = nullptr;
  TRY(sc.alloc(&nbc, (size_t)ne + 1));
  TRY(sc.alloc(&nbs, (size_t)ne + 1));
  TRY(sc.alloc(&d_over, 1));
  CUDA_TRY(cudaMemsetAsync(nbc, 0, sizeof(unsigned) * (ne + 1), st));
  CUDA_TRY(cudaMemsetAsync(d_over, 0, sizeof(int), st));
  k_nb_count<<<nblk(ne), kBlock, 0, st>>>(ne, h->d_nie, h->d_cin_start, h->d_cin, nbc, d_over);
  TRY(exclusive_scan(sc, nbc, nbs, (long long)ne + 1, st));
  unsigned nnz = 0;
  int over = 0;
  CUDA_TRY(cudaMemcpyAsync(&nnz, nbs + ne, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(&over, d_over, sizeof(int), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (over) return set_error(FIERRO_ENOTSUP, "topology: an element has more than %d neighbours", kMaxNb);
  TRY(hd::dalloc(h, &h->d_eie, (size_t)nnz));
  h->nnz_eie = (int64_t)nnz;
  k_to_int<<<nblk(ne + 1), kBlock, 0, st>>>(ne + 1, nbs, h->d_eie_start);
  k_nb_fill<<<nblk(ne), kBlock, 0, st>>>(ne, h->d_nie, h->d_cin_start, h->d_cin, h->d_eie_start, h->d_eie);
  // ---- boundary node masks
  std::vector<Bc> hb((size_t)num_bcs);
  for (int64_t s = 0; s < num_bcs; ++s)
    hb[s] = {bcs[s].surface, (int)bc_mask_bits(bcs[s].hydro_bc, bcs[s].surface, 3), bcs[s].value};
  Bc* d_bcs = nullptr;
  unsigned* m32 = nullptr;
  TRY(sc.alloc(&d_bcs, hb.size()));
  TRY(sc.alloc(&m32, (size_t)nn));
  if (!hb.empty()) CUDA_TRY(cudaMemcpyAsync(d_bcs, hb.data(), sizeof(Bc) * hb.size(), cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemsetAsync(m32, 0, sizeof(unsigned) * nn, st));
  k_patches<<<nblk((long long)ne * 6), kBlock, 0, st>>>(ne, h->d_nie, h->d_cin_start, h->d_cin, xyz, node_int2ext,
                                                         d_bcs, (int)num_bcs, m32);
  k_mask_u8<<<nblk(nn), kBlock, 0, st>>>(nn, m32, h->d_bc);
  CUDA_TRY(cudaGetLastError());
  // ---- the host keeps the renumbering (staged transfers, adjoint I/O)
  std::vector<int32_t> tmp((size_t)std::max(nn, ne));
  HostTopo& t = h->topo;
  t.nn = nn;
  t.ne = ne;
  CUDA_TRY(cudaMemcpyAsync(tmp.data(), node_int2ext, sizeof(int) * nn, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  t.node_int2ext.assign(tmp.begin(), tmp.begin() + nn);
  CUDA_TRY(cudaMemcpyAsync(tmp.data(), elem_int2ext, sizeof(int) * ne, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  t.elem_int2ext.assign(tmp.begin(), tmp.begin() + ne);
  return FIERRO_OK;
}

}  // namespace topo
}  // namespace fierro
