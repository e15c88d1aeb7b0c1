// The persistent solver handle and the helpers that build per-launch argument
// records from it; shared by the C ABI (sgh_capi.cpp) and the discrete adjoint
// (sgh_adjoint.cpp).  Internal, not part of include/fierro_sgh.h.
#ifndef FIERRO_SGH_HANDLE_H
#define FIERRO_SGH_HANDLE_H

#include <algorithm>
#include <vector>

#include <cuda_runtime.h>

#include "fierro_sgh.h"
#include "sgh_device.h"
#include "sgh_internal.h"
#include "sgh_xfer.h"

#define CUDA_TRY(expr)                                                                            \
  do {                                                                                            \
    cudaError_t err_ = (expr);                                                                    \
    if (err_ != cudaSuccess)                                                                      \
      return set_error(err_ == cudaErrorMemoryAllocation ? FIERRO_ENOMEM : FIERRO_ECUDA, "%s: %s", \
                       #expr, cudaGetErrorString(err_));                                          \
  } while (0)

#define TRY(expr)          \
  do {                     \
    int rc_ = (expr);      \
    if (rc_) return rc_;   \
  } while (0)

namespace fierro {
struct AdjState;
struct AdjBranches;
struct OutputState;
struct RzKernelSet;
}

struct fierro_sgh {
  fierro::HostTopo topo;
  int64_t nn = 0, ne = 0;
  int nmat = 0;
  int fp_mode = FIERRO_FP_EXACT;
  const fierro::KernelSet* ks = nullptr;
  fierro::LoopParams lp{};
  int rk_num_stages = 2;
  double dt_start = 1e-5;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::vector<void*> allocations;
  size_t dev_bytes = 0;
  // mesh
  int *d_nie = nullptr, *d_cin_start = nullptr, *d_cin = nullptr, *d_eie_start = nullptr, *d_eie = nullptr;
  int* d_mat = nullptr;
  unsigned char* d_bc = nullptr;
  double* d_qtab = nullptr;
  // state
  double *d_node_mass = nullptr, *d_elem_mass = nullptr, *d_gamma = nullptr, *d_csmin = nullptr;
  double* d_node_rm = nullptr;  // 1 / node mass of the uploaded state (FMA-mode node update, hex meshes)
  double* d_x[2][3] = {};
  double* d_v[2][3] = {};
  double* d_h[3] = {};
  double *d_den = nullptr, *d_pres = nullptr, *d_sspd = nullptr, *d_vol = nullptr;
  double* d_div[2] = {};  // see sgh_device.h: read by stage parity q, written at q^1
  double* d_sie[2] = {};
  double *d_bmat = nullptr, *d_force = nullptr;
  long long* d_cfl = nullptr;
  int ncfl = 0;  // CFL partials: one per element block
  // threads per block of the element, force and node kernels (small_mesh_block)
  int blk_elem = fierro::kElemBlock, blk_force = fierro::kForceBlock, blk_node = fierro::kNodeBlock;
  fierro::Ctrl* d_ctrl = nullptr;
  double *d_energy_part = nullptr, *d_energy_out = nullptr;
  // pinned double buffer for permuted transfers
  double* h_stage[2] = {};
  cudaEvent_t stage_ev[2] = {};
  size_t stage_elems = 0;
  // loop position
  int base = 0;          // bin holding the state uploaded by set_state
  long long enq_cycles = 0;  // cycles enqueued since set_state
  int stage = 0;         // next RK stage of the current cycle (stage stepping)
  bool has_state = false;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  fierro::AdjState* adj = nullptr;  // discrete-adjoint tape and checkpoints (sgh_adjoint.cpp)
  fierro::AdjBranches* adj_br = nullptr;  // branch record of the frozen-branch forward (sgh_adjoint.cpp)
  // direct transfers (sgh_xfer.cu): caller -> internal maps and the validation word
  bool direct_host = false;
  int* d_node_ext2int = nullptr;
  int* d_elem_ext2int = nullptr;
  int* d_node_int2ext = nullptr;
  int* d_elem_int2ext = nullptr;
  fierro::XferStatus* d_xfer = nullptr;
  int64_t nnz_eie = 0;  // neighbour-list entries
  fierro::OutputState* out = nullptr;  // graphics dumps (sgh_output.cpp)
  // strength materials (sgh_user_mat.cuh): two stress bins [9][ne] and the
  // element state variables [nsv][ne] (sized by set_state, owned separately)
  bool strength = false;   // some material has strength_type 1 or 2
  bool has_hyper = false;  // some material has strength_type 2
  int* d_stype = nullptr;
  double* d_stress[2] = {};
  double* d_statev = nullptr;
  int64_t nsv = 0;
  // 2D-RZ handles (num_dims == 2, sgh_rz.cpp): quad kernels, the stage-start
  // radius and extensive mass per node, the boundary nodes for the axis fix
  int dims = 3;
  double tiny = 1.0e-12;
  const fierro::RzKernelSet* rks = nullptr;
  double* d_rad = nullptr;
  double* d_node_ext = nullptr;
  int* d_axis = nullptr;
  int* d_axis_nin_start = nullptr;
  int* d_axis_nin = nullptr;
  int naxis = 0;
  // host-side fault injection: FIERRO_FAIL_ALLOC_AFTER=n makes the handle's
  // device allocations after the first n fail as if the device were full
  int64_t alloc_limit = -1;
  int64_t alloc_count = 0;
};

namespace fierro {

namespace hd {

template <typename T>
int dalloc(fierro_sgh* h, T** p, size_t count) {
  void* q = nullptr;
  size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
  if (h->alloc_limit >= 0 && h->alloc_count >= h->alloc_limit)
    return set_error(FIERRO_ENOMEM, "cudaMalloc(%zu bytes): injected failure after %lld allocations", bytes,
                     (long long)h->alloc_count);
  h->alloc_count++;
  cudaError_t err = cudaMalloc(&q, bytes);
  if (err != cudaSuccess)
    return set_error(FIERRO_ENOMEM, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(err));
  h->allocations.push_back(q);
  h->dev_bytes += bytes;
  *p = static_cast<T*>(q);
  return FIERRO_OK;
}

int upload_raw(fierro_sgh* h, void* dst, const void* src, size_t bytes);
// Permuted upload through the pinned double buffer: dst[i] = src[map[i]*stride + off].
int upload_gather(fierro_sgh* h, double* dst, const double* src, const std::vector<int64_t>& map,
                  size_t stride, size_t off, int* slot);
// Permuted download: out[map[i]*stride + off] = src[i].
int download_scatter(fierro_sgh* h, double* out, const double* src, const std::vector<int64_t>& map,
                     size_t stride, size_t off);
int check_status(fierro_sgh* h);
int cycles_done(fierro_sgh* h, long long* cyc);
ForceArgs force_args(fierro_sgh* h, int rb, int q);
NodeArgs node_args(fierro_sgh* h, int c, double alpha);
ElemArgs elem_args(fierro_sgh* h, int cur_bin, int c, double alpha, int div_out);
// The force and element records of RK stage s of a cycle whose start state is in
// bin c, with the stress bins of a strength handle.
ForceArgs stage_force_args(fierro_sgh* h, int c, int s);
ElemArgs stage_elem_args(fierro_sgh* h, int c, int s);

// Bins at a cycle boundary after `done` executed cycles: state bin and start bin.
inline int bin_now(const fierro_sgh* h, long long cycles_done) { return (int)((h->base + cycles_done) & 1); }
inline double stage_alpha(const fierro_sgh* h, int s) {
  return 1.0 / ((double)h->rk_num_stages - (double)s);  // sgh_solve.cpp:353
}
// Divergence buffer a stage reads: the parity of the number of stages run since
// set_state, which for stage s of a cycle with bin parity c is (c*S + s) & 1.
inline int div_parity(const fierro_sgh* h, int c, int s) { return (c * h->rk_num_stages + s) & 1; }

}  // namespace hd

// Frees the adjoint's device memory (no-op without one).
void adj_release(fierro_sgh* h);
// Frees the branch record of the frozen-branch forward (no-op without one).
void adj_branches_release(fierro_sgh* h);

// Graphics dumps (sgh_output.cpp).
void output_release(fierro_sgh* h);
xfer::SnapArgs output_snap_args(fierro_sgh* h, int bin, int force);
int output_before_cycle(fierro_sgh* h, long long cycles_enqueued);
int output_after_cycle(fierro_sgh* h);
void output_reset(fierro_sgh* h);
// Re-instantiates the per-parity cycle graphs (with or without the snapshot).
int rebuild_graphs(fierro_sgh* h);

}  // namespace fierro

#endif
