// fierro_sgh_validate: checks the device topology of a handle against the
// invariants the cycle kernels rely on, on the GPU, without trusting it for any
// access: every index is range-checked before it is used, and a failing check
// only records the smallest offending index.  It stands in for a memory checker
// (the kernels never index outside these arrays when the checks pass) and tests
// the GPU topology builder (sgh_topo.cu) on real meshes.
//
// Checks (npe = 8 for hexes, 4 for quads):
//   NIE      every element's nodes are node ids, pairwise distinct
//   CSR      the corner CSR is monotone, starts at 0 and ends at ne*npe
//   CORNER   every corner listed at node n is a corner id whose element has n at
//            that local node, and each node's corners come in strictly
//            increasing caller element order (the reference's summation order,
//            mesh.h:218-241) -- with the count, every corner appears exactly once
//   NEIGHBOUR every neighbour is another element sharing at least one node
//   BC       boundary masks use only the velocity components of the mesh
//   AXIS     (2D-RZ) boundary-node and edge-neighbour ids are node ids
#include <climits>
#include <cstdint>

#include "sgh_handle.h"

namespace fierro {
namespace {

enum Check { NIE = 0, CSR, CORNER, NEIGHBOUR, BC, AXIS, NCHECK };
const char* const kCheckName[NCHECK] = {"element nodes", "corner CSR offsets", "corner lists",
                                        "neighbour lists", "boundary masks", "axis lists"};

struct Report {
  unsigned int flags;
  int pad;
  long long first[NCHECK];
};

struct ValArgs {
  int nn, ne, npe, dims, naxis;
  long long nnz, nnz_axis;
  const int* nie;
  const int* cin_start;
  const int* cin;
  const int* eie_start;
  const int* eie;
  const unsigned char* bc;
  const int* elem_int2ext;  // may be null
  const int* axis;
  const int* axis_nin_start;
  const int* axis_nin;
  Report* rep;
};

__device__ void fail(Report* r, int which, long long idx) {
  atomicOr(&r->flags, 1u << which);
  atomicMin(&r->first[which], idx);
}

__device__ bool elem_has(const ValArgs& a, int e, int n) {
  for (int l = 0; l < a.npe; ++l)
    if (a.nie[(size_t)e * a.npe + l] == n) return true;
  return false;
}

__global__ void k_val_elems(const ValArgs a) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.ne) return;
  bool ok = true;
  for (int l = 0; l < a.npe; ++l) {
    const int n = a.nie[(size_t)e * a.npe + l];
    if (n < 0 || n >= a.nn) ok = false;
    for (int k = 0; k < l; ++k)
      if (a.nie[(size_t)e * a.npe + k] == n) ok = false;
  }
  if (!ok) {
    fail(a.rep, NIE, e);
    return;
  }
  const int k0 = a.eie_start[e], k1 = a.eie_start[e + 1];
  if (k0 < 0 || k1 < k0 || (long long)k1 > a.nnz) {
    fail(a.rep, NEIGHBOUR, e);
    return;
  }
  for (int k = k0; k < k1; ++k) {
    const int o = a.eie[k];
    if (o < 0 || o >= a.ne || o == e) {
      fail(a.rep, NEIGHBOUR, e);
      return;
    }
    bool shares = false;
    for (int l = 0; l < a.npe && !shares; ++l) shares = elem_has(a, o, a.nie[(size_t)e * a.npe + l]);
    if (!shares) {
      fail(a.rep, NEIGHBOUR, e);
      return;
    }
  }
}

__global__ void k_val_nodes(const ValArgs a) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= a.nn) return;
  const long long total = (long long)a.ne * a.npe;
  const int c0 = a.cin_start[n], c1 = a.cin_start[n + 1];
  if (c0 < 0 || c1 < c0 || c1 > total || (n == 0 && c0 != 0) || (n == a.nn - 1 && c1 != total)) {
    fail(a.rep, CSR, n);
    return;
  }
  const int shift = a.npe == 8 ? 3 : 2;
  long long prev = -1;
  for (int c = c0; c < c1; ++c) {
    const int cid = a.cin[c];
    if (cid < 0 || (long long)cid >= total || a.nie[cid] != n) {
      fail(a.rep, CORNER, n);
      return;
    }
    const int e = cid >> shift;
    const long long ext = a.elem_int2ext ? (long long)a.elem_int2ext[e] : (long long)e;
    if (a.elem_int2ext && ext <= prev) {
      fail(a.rep, CORNER, n);
      return;
    }
    prev = ext;
  }
  const unsigned allowed = a.dims == 2 ? 3u : 7u;
  if (a.bc[n] & ~allowed) fail(a.rep, BC, n);
}

__global__ void k_val_axis(const ValArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.naxis) return;
  const int n = a.axis[i];
  const int k0 = a.axis_nin_start[i], k1 = a.axis_nin_start[i + 1];
  bool ok = n >= 0 && n < a.nn && k0 >= 0 && k1 >= k0 && (long long)k1 <= a.nnz_axis;
  for (int k = k0; ok && k < k1; ++k) ok = a.axis_nin[k] >= 0 && a.axis_nin[k] < a.nn && a.axis_nin[k] != n;
  if (!ok) fail(a.rep, AXIS, i);
}

}  // namespace
}  // namespace fierro

using namespace fierro;

extern "C" int fierro_sgh_validate(fierro_sgh* h) {
  clear_error();
  if (!h) return set_error(FIERRO_EINVAL, "handle is NULL");
  Report init{};
  for (int k = 0; k < NCHECK; ++k) init.first[k] = LLONG_MAX;
  Report* d_rep = nullptr;
  CUDA_TRY(cudaMalloc(&d_rep, sizeof(Report)));
  cudaError_t err = cudaMemcpyAsync(d_rep, &init, sizeof(Report), cudaMemcpyHostToDevice, h->stream);
  ValArgs a{};
  a.nn = (int)h->nn;
  a.ne = (int)h->ne;
  a.npe = h->dims == 2 ? 4 : 8;
  a.dims = h->dims;
  a.nnz = h->nnz_eie;
  a.nie = h->d_nie;
  a.cin_start = h->d_cin_start;
  a.cin = h->d_cin;
  a.eie_start = h->d_eie_start;
  a.eie = h->d_eie;
  a.bc = h->d_bc;
  a.elem_int2ext = h->d_elem_int2ext;
  a.axis = h->d_axis;
  a.axis_nin_start = h->d_axis_nin_start;
  a.axis_nin = h->d_axis_nin;
  a.naxis = h->naxis;
  a.nnz_axis = (long long)h->topo.axis_nin.size();
  a.rep = d_rep;
  const int bs = 256;
  if (err == cudaSuccess) {
    k_val_elems<<<(unsigned)((a.ne + bs - 1) / bs), bs, 0, h->stream>>>(a);
    k_val_nodes<<<(unsigned)((a.nn + bs - 1) / bs), bs, 0, h->stream>>>(a);
    if (a.naxis > 0) k_val_axis<<<(unsigned)((a.naxis + bs - 1) / bs), bs, 0, h->stream>>>(a);
    err = cudaGetLastError();
  }
  Report rep{};
  if (err == cudaSuccess) err = cudaMemcpyAsync(&rep, d_rep, sizeof(Report), cudaMemcpyDeviceToHost, h->stream);
  if (err == cudaSuccess) err = cudaStreamSynchronize(h->stream);
  cudaFree(d_rep);
  if (err != cudaSuccess) return set_error(FIERRO_ECUDA, "validate: %s", cudaGetErrorString(err));
  for (int k = 0; k < NCHECK; ++k)
    if (rep.flags & (1u << k))
      return set_error(FIERRO_EINVAL, "validate: %s fail their check (first index %lld)", kCheckName[k],
                       rep.first[k]);
  return FIERRO_OK;
}
