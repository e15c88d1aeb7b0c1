// Batched ensemble: many independent SGH problems in one device layout.
//
// Instance i owns nodes [node_off[i], node_off[i+1]) and elements
// [elem_off[i], elem_off[i+1]); element ranges are padded to whole blocks of the
// element kernel so each block (and its CFL partial minimum) belongs to one
// instance.  Every launch of a cycle covers all instances; the kernels find an
// item's instance through the per-element / per-node instance maps and read that
// instance's dt, activity and CFL number from per-instance tables.  Within an
// instance nothing changes: same numbering rules, summation orders and
// arithmetic as the single-problem handle, so results agree bit for bit.
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "fierro_sgh.h"
#include "sgh_device.h"
#include "sgh_internal.h"

using namespace fierro;

#define CUDA_TRY(expr)                                                                            \
  do {                                                                                            \
    cudaError_t err_ = (expr);                                                                    \
    if (err_ != cudaSuccess)                                                                      \
      return set_error(err_ == cudaErrorMemoryAllocation ? FIERRO_ENOMEM : FIERRO_ECUDA, "%s: %s", \
                       #expr, cudaGetErrorString(err_));                                          \
  } while (0)

#define TRY(expr)        \
  do {                   \
    int rc_ = (expr);    \
    if (rc_) return rc_; \
  } while (0)

struct fierro_batch {
  int64_t n = 0;
  int rk_num_stages = 2;
  double fuzz = 1e-16, small = 1e-8;
  const KernelSet* ks = nullptr;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::vector<HostTopo> topo;
  std::vector<int64_t> node_off, elem_off, mat_off;
  std::vector<int> part_start;
  std::vector<LoopParams> lps;
  std::vector<double> dt_start;
  std::vector<char> has_state;
  int64_t NN = 0, NE = 0;
  int nparts = 0;
  bool started = false;
  long long enq_cycles = 0;
  std::vector<void*> allocations;
  size_t dev_bytes = 0;
  int *d_nie = nullptr, *d_cin_start = nullptr, *d_cin = nullptr, *d_eie_start = nullptr, *d_eie = nullptr;
  int *d_mat = nullptr, *d_inst_e = nullptr, *d_inst_n = nullptr, *d_part_start = nullptr;
  unsigned char* d_bc = nullptr;
  double *d_qtab = nullptr, *d_dt_cfl = nullptr;
  LoopParams* d_lps = nullptr;
  double *d_node_mass = nullptr, *d_elem_mass = nullptr, *d_gamma = nullptr, *d_csmin = nullptr;
  double* d_node_rm = nullptr;  // 1 / node mass (FMA-mode node update), formed at the first run
  double* d_x[2][3] = {};
  double* d_v[2][3] = {};
  double* d_h[3] = {};
  double *d_den = nullptr, *d_pres = nullptr, *d_sspd = nullptr, *d_vol = nullptr;
  double* d_div[2] = {};
  double* d_sie[2] = {};
  double *d_bmat = nullptr, *d_force = nullptr;
  long long* d_cfl = nullptr;
  Ctrl* d_ctrl = nullptr;
  unsigned int* d_sync = nullptr;  // fused stage: arrival counter, generation, timeout status
  cudaError_t capture_err = cudaSuccess;
  double* h_stage = nullptr;
  size_t stage_elems = 0;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  // launch shape of the cycle kernels (fierro_batch_set_shape / fierro_batch_autotune)
  fierro_batch_shape shape{kForceBlock, kNodeBlock, kElemBlock, 0, 0};
  int sm_count = 0;
  std::vector<fierro_batch_shape> tune_shapes;
  std::vector<double> tune_ms;
};

namespace {

template <typename T>
int balloc(fierro_batch* b, T** p, size_t count) {
  void* q = nullptr;
  size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
  cudaError_t err = cudaMalloc(&q, bytes);
  if (err != cudaSuccess) return set_error(FIERRO_ENOMEM, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(err));
  b->allocations.push_back(q);
  b->dev_bytes += bytes;
  *p = static_cast<T*>(q);
  return FIERRO_OK;
}

template <typename T>
int put(fierro_batch* b, T* dst, const std::vector<T>& src) {
  if (src.empty()) return FIERRO_OK;
  CUDA_TRY(cudaMemcpyAsync(dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return FIERRO_OK;
}

// dst[off + k] = src[map[k] * stride + sub] through the pinned staging buffer.
int gather_up(fierro_batch* b, double* dst, int64_t off, const double* src, const std::vector<int64_t>& map,
              size_t stride, size_t sub) {
  const int64_t n = (int64_t)map.size();
  for (int64_t k = 0; k < n; ++k) b->h_stage[k] = src[(size_t)map[k] * stride + sub];
  CUDA_TRY(cudaMemcpyAsync(dst + off, b->h_stage, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return FIERRO_OK;
}

int scatter_down(fierro_batch* b, double* out, const double* src, int64_t off, const std::vector<int64_t>& map,
                 size_t stride, size_t sub) {
  const int64_t n = (int64_t)map.size();
  CUDA_TRY(cudaMemcpyAsync(b->h_stage, src + off, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  for (int64_t k = 0; k < n; ++k) out[(size_t)map[k] * stride + sub] = b->h_stage[k];
  return FIERRO_OK;
}

// A persistent grid fills every SM `shape.persistent` times over with the
// kernel's resident blocks at this block size; 0 = one block per tile.
int persistent_grid(const fierro_batch* b, int kernel, int block) {
  if (!b->shape.persistent) return 0;
  return b->sm_count * b->ks->batch_max_blocks(kernel, block) * b->shape.persistent;
}

// A fused stage whose grid barrier gave up waiting (never expected: the launch
// is cooperative) leaves results that cannot be trusted: report it, and reset
// the barrier for the next launch.  Call with the stream idle.
int check_sync(fierro_batch* b) {
  if (!b->shape.fused_stage) return FIERRO_OK;
  unsigned int st = 0;
  CUDA_TRY(cudaMemcpy(&st, b->d_sync + 2, sizeof(st), cudaMemcpyDeviceToHost));
  if (st == 0) return FIERRO_OK;
  CUDA_TRY(cudaMemset(b->d_sync, 0, 3 * sizeof(unsigned int)));
  return set_error(FIERRO_ETIMEDOUT, "batch: a fused stage's grid barrier timed out");
}

// The fused stage's grid: every resident block of the cooperative kernel at the
// element block size, at most one per element tile.  Failure-detection test hook
// (host side, like FIERRO_FAIL_ALLOC_AFTER): FIERRO_FUSED_OVERSUBSCRIBE=k > 1
// launches k times the resident blocks without the cooperative attribute, so the
// grid barrier cannot complete and every block's bounded wait runs out.
int fused_oversubscribe() {
  const char* env = std::getenv("FIERRO_FUSED_OVERSUBSCRIBE");
  const int k = env ? std::atoi(env) : 0;
  return k > 1 && k <= 16 ? k : 0;
}
int fused_grid(const fierro_batch* b) {
  const long long tiles = b->NE / b->shape.elem_block;
  const long long resident = (long long)b->sm_count * b->ks->fused_max_blocks(b->shape.elem_block);
  if (const int k = fused_oversubscribe()) return (int)std::max<long long>(1, resident * k);
  return (int)std::max<long long>(1, std::min(tiles, resident));
}

ForceArgs b_force(fierro_batch* b, int rb, int q) {
  ForceArgs a{};
  a.ne = (int)b->NE;
  a.nie = b->d_nie;
  a.eie_start = b->d_eie_start;
  a.eie = b->d_eie;
  a.mat = b->d_mat;
  a.qtab = b->d_qtab;
  a.bmat = b->d_bmat;
  a.u = b->d_v[rb][0];
  a.v = b->d_v[rb][1];
  a.w = b->d_v[rb][2];
  a.den = b->d_den;
  a.pres = b->d_pres;
  a.sspd = b->d_sspd;
  a.vol = b->d_vol;
  a.div = b->d_div[q];
  a.force = b->d_force;
  a.ctrl = b->d_ctrl;
  a.inst = b->d_inst_e;
  a.fuzz = b->fuzz;
  a.small = b->small;
  a.block = b->shape.force_block;
  a.grid = persistent_grid(b, 0, b->shape.force_block);
  return a;
}

NodeArgs b_node(fierro_batch* b, int c, double alpha) {
  NodeArgs a{};
  a.nn = (int)b->NN;
  a.ne = (int)b->NE;
  a.cin_start = b->d_cin_start;
  a.cin = b->d_cin;
  a.force = b->d_force;
  a.node_mass = b->d_node_mass;
  a.node_rm = b->d_node_rm;
  a.bc_mask = b->d_bc;
  a.u0 = b->d_v[c][0];
  a.v0 = b->d_v[c][1];
  a.w0 = b->d_v[c][2];
  a.x0 = b->d_x[c][0];
  a.y0 = b->d_x[c][1];
  a.z0 = b->d_x[c][2];
  a.u1 = b->d_v[c ^ 1][0];
  a.v1 = b->d_v[c ^ 1][1];
  a.w1 = b->d_v[c ^ 1][2];
  a.x1 = b->d_x[c ^ 1][0];
  a.y1 = b->d_x[c ^ 1][1];
  a.z1 = b->d_x[c ^ 1][2];
  a.hx = b->d_h[0];
  a.hy = b->d_h[1];
  a.hz = b->d_h[2];
  a.ctrl = b->d_ctrl;
  a.inst = b->d_inst_n;
  a.rk_alpha = alpha;
  a.block = b->shape.node_block;
  a.grid = persistent_grid(b, 1, b->shape.node_block);
  return a;
}

ElemArgs b_elem(fierro_batch* b, int cur_bin, int c, double alpha, int div_out) {
  ElemArgs a{};
  a.ne = (int)b->NE;
  a.nie = b->d_nie;
  a.x = b->d_x[cur_bin][0];
  a.y = b->d_x[cur_bin][1];
  a.z = b->d_x[cur_bin][2];
  a.u = b->d_v[cur_bin][0];
  a.v = b->d_v[cur_bin][1];
  a.w = b->d_v[cur_bin][2];
  a.hx = b->d_h[0];
  a.hy = b->d_h[1];
  a.hz = b->d_h[2];
  a.force = b->d_force;
  a.mass = b->d_elem_mass;
  a.sie0 = b->d_sie[c];
  a.sie1 = b->d_sie[c ^ 1];
  a.gamma = b->d_gamma;
  a.csmin = b->d_csmin;
  a.den = b->d_den;
  a.pres = b->d_pres;
  a.sspd = b->d_sspd;
  a.vol = b->d_vol;
  a.div = b->d_div[div_out];
  a.bmat = b->d_bmat;
  a.cfl_part = b->d_cfl;
  a.ctrl = b->d_ctrl;
  a.inst = b->d_inst_e;
  a.dt_cfl_tab = b->d_dt_cfl;
  a.rk_alpha = alpha;
  a.fuzz = b->fuzz;
  a.block = b->shape.elem_block;
  a.grid = persistent_grid(b, 2, b->shape.elem_block);
  return a;
}

void b_cycle(fierro_batch* b, int c) {
  DtArgs d{};
  d.cfl_part = b->d_cfl;
  d.nparts = b->nparts;
  d.ctrl = b->d_ctrl;
  d.part_start = b->d_part_start;
  d.lps = b->d_lps;
  d.ninst = (int)b->n;
  b->ks->dt(d, b->stream);
  const int S = b->rk_num_stages;
  for (int s = 0; s < S; ++s) {
    const double alpha = 1.0 / ((double)S - (double)s);  // sgh_solve.cpp:353
    const int rb = (s == 0) ? c : (c ^ 1);
    const int q = (c * S + s) & 1;
    if (b->shape.fused_stage) {
      // one cooperative launch for the stage, its barrier's arrival count reset first
      ForceArgs fa = b_force(b, rb, q);
      NodeArgs na = b_node(b, c, alpha);
      ElemArgs ea = b_elem(b, c ^ 1, c, alpha, q ^ 1);
      fa.grid = na.grid = ea.grid = 0;
      const StageSync sync{b->d_sync, b->d_sync + 1, b->d_sync + 2};
      cudaError_t err = cudaMemsetAsync(b->d_sync, 0, sizeof(unsigned int), b->stream);
      if (err == cudaSuccess)
        err = b->ks->stage_fused(fa, na, ea, (s == S - 1) ? 1 : 0, sync, fused_grid(b), fused_oversubscribe() ? 0 : 1,
                                 b->stream);
      if (err != cudaSuccess && b->capture_err == cudaSuccess) b->capture_err = err;
      continue;
    }
    b->ks->force(b_force(b, rb, q), b->stream);
    b->ks->node(b_node(b, c, alpha), b->stream);
    b->ks->elem(b_elem(b, c ^ 1, c, alpha, q ^ 1), (s == S - 1) ? 1 : 0, b->stream);
  }
  b->ks->end_batch(b->d_ctrl, b->d_lps, (int)b->n, b->stream);
}

constexpr int kMinBatchBlock = 32;

bool shape_valid(const fierro_batch_shape& sh) {
  auto ok = [](int b, int hi) { return b >= kMinBatchBlock && b <= hi && (b & (b - 1)) == 0; };
  return ok(sh.force_block, kForceBlock) && ok(sh.node_block, 1024) && ok(sh.elem_block, kElemBlock) &&
         sh.persistent >= 0 && sh.persistent <= 8 && (sh.fused_stage == 0 || sh.fused_stage == 1);
}

// Makes `sh` the batch's launch shape: the per-instance CFL partial ranges in
// tiles of sh.elem_block elements, and the two per-parity cycle graphs.
int apply_shape(fierro_batch* b, const fierro_batch_shape& sh) {
  if (!shape_valid(sh))
    return set_error(FIERRO_EINVAL, "batch shape: blocks must be powers of two, force 32..%d, node 32..1024, "
                     "element 32..%d, persistent 0..8 fills of the SMs, fused_stage 0 or 1", kForceBlock, kElemBlock);
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  b->shape = sh;
  for (size_t i = 0; i < b->part_start.size(); ++i)
    b->part_start[i] = (int)(b->elem_off[i] / sh.elem_block);
  b->nparts = b->part_start.back();
  TRY(put(b, b->d_part_start, b->part_start));
  for (int c = 0; c < 2; ++c) {
    if (b->graph[c]) {
      cudaGraphExecDestroy(b->graph[c]);
      b->graph[c] = nullptr;
    }
    cudaGraph_t g = nullptr;
    b->capture_err = cudaSuccess;
    CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    b_cycle(b, c);
    cudaError_t err = cudaStreamEndCapture(b->stream, &g);
    if (err == cudaSuccess && b->capture_err != cudaSuccess) err = b->capture_err;
    if (err == cudaSuccess) err = cudaGraphInstantiate(&b->graph[c], g, 0);
    if (g) cudaGraphDestroy(g);
    if (err != cudaSuccess) return set_error(FIERRO_ECUDA, "batch cycle graph: %s", cudaGetErrorString(err));
  }
  return FIERRO_OK;
}

int create_impl(fierro_batch* b, const fierro_batch_instance* inst, int64_t n, int fp_mode, void* stream) {
  if (!inst || n < 1) return set_error(FIERRO_EINVAL, "batch: need at least one instance");
  if (n > (1 << 24)) return set_error(FIERRO_EINVAL, "batch: too many instances");
  if (fp_mode != FIERRO_FP_EXACT && fp_mode != FIERRO_FP_FMA) return set_error(FIERRO_EINVAL, "fp_mode %d unknown", fp_mode);
  b->n = n;
  b->ks = (fp_mode == FIERRO_FP_EXACT) ? &kernels_exact() : &kernels_fma();
  const fierro_sgh_params& p0 = inst[0].params;
  b->rk_num_stages = (int)p0.rk_num_stages;
  b->fuzz = p0.fuzz;
  b->small = p0.small;
  if (p0.rk_num_stages < 1 || p0.rk_num_stages > 8) return set_error(FIERRO_EINVAL, "batch: rk_num_stages out of range");
  b->topo.resize((size_t)n);
  b->node_off.assign((size_t)n + 1, 0);
  b->elem_off.assign((size_t)n + 1, 0);
  b->mat_off.assign((size_t)n + 1, 0);
  b->part_start.assign((size_t)n + 1, 0);
  b->lps.resize((size_t)n);
  b->dt_start.resize((size_t)n);
  b->has_state.assign((size_t)n, 0);
  for (int64_t i = 0; i < n; ++i) {
    const fierro_batch_instance& I = inst[i];
    const fierro_sgh_params& p = I.params;
    if (p.rk_num_stages != p0.rk_num_stages || p.fuzz != p0.fuzz || p.small != p0.small || p.tiny != p0.tiny)
      return set_error(FIERRO_EINVAL, "batch: instance %lld: rk_num_stages, fuzz, tiny and small must match", (long long)i);
    if (p.graphics_cyc_ival < 1 || !(p.dt_cfl > 0) || !(p.dt_max > 0) || !(p.dt_min > 0) || !(p.dt_start > 0))
      return set_error(FIERRO_EINVAL, "batch: instance %lld: bad time-step controls", (long long)i);
    if (I.num_materials < 1 || !I.materials) return set_error(FIERRO_EINVAL, "batch: instance %lld: no material", (long long)i);
    for (int64_t m = 0; m < I.num_materials; ++m)
      if (I.materials[m].eos_model != 0 || I.materials[m].strength_type != 0)
        return set_error(FIERRO_ENOTSUP, "batch: instance %lld: only ideal gas without strength", (long long)i);
    if (mesh_dims(&I.mesh) == 2)
      return set_error(FIERRO_ENOTSUP, "batch: instance %lld is a 2D-RZ mesh (hex meshes only)", (long long)i);
    int rc = build_topology(&I.mesh, I.boundaries, I.num_bcs, true, &b->topo[i]);
    if (rc) {
      std::string msg = fierro_last_error();
      return set_error(rc, "batch: instance %lld: %s", (long long)i, msg.c_str());
    }
    const int64_t ne_pad = (I.mesh.num_elems + kElemBlock - 1) / kElemBlock * kElemBlock;
    b->node_off[i + 1] = b->node_off[i] + I.mesh.num_nodes;
    b->elem_off[i + 1] = b->elem_off[i] + ne_pad;
    b->mat_off[i + 1] = b->mat_off[i] + I.num_materials;
    b->part_start[i + 1] = (int)(b->elem_off[i + 1] / kElemBlock);  // per default block; see apply_shape
    b->lps[i] = LoopParams{p.time_final, p.dt_max, p.dt_min, p.dt_cfl, p.graphics_dt_ival, p.fuzz, p.small,
                           p.graphics_cyc_ival};
    b->dt_start[i] = p.dt_start;
  }
  b->NN = b->node_off[n];
  b->NE = b->elem_off[n];
  b->nparts = b->part_start[n];
  if (b->NE * 8 >= (int64_t)INT32_MAX || b->NN >= (int64_t)INT32_MAX)
    return set_error(FIERRO_EINVAL, "batch too large for 32-bit device indices");
  // concatenated mesh arrays (global ids)
  const int64_t NN = b->NN, NE = b->NE;
  std::vector<int32_t> nie((size_t)NE * 8, 0), cin_start((size_t)NN + 1, 0), cin, eie_start((size_t)NE + 1, 0), eie;
  std::vector<int32_t> mat((size_t)NE, 0), inst_e((size_t)NE, 0), inst_n((size_t)NN, 0);
  std::vector<uint8_t> bc((size_t)NN, 0);
  std::vector<double> qtab((size_t)b->mat_off[n] * 4), dtc((size_t)n);
  cin.reserve((size_t)NE * 8);
  for (int64_t i = 0; i < n; ++i) {
    const HostTopo& t = b->topo[i];
    const int64_t no = b->node_off[i], eo = b->elem_off[i];
    for (int64_t e = 0; e < t.ne * 8; ++e) nie[(size_t)eo * 8 + e] = (int32_t)(t.nie[e] + no);
    for (int64_t e = eo; e < b->elem_off[i + 1]; ++e) inst_e[e] = (e - eo < t.ne) ? (int32_t)i : (int32_t)(-i - 1);
    for (int64_t k = 0; k < t.nn; ++k) {
      cin_start[no + k + 1] = (int32_t)(t.cin_start[k + 1] - t.cin_start[k]);
      inst_n[no + k] = (int32_t)i;
      bc[no + k] = t.bc_mask[k];
    }
    for (int32_t c : t.cin) cin.push_back((int32_t)(c + eo * 8));
    for (int64_t e = 0; e < t.ne; ++e) eie_start[eo + e + 1] = t.eie_start[e + 1] - t.eie_start[e];
    for (int32_t o : t.eie) eie.push_back((int32_t)(o + eo));
    const fierro_batch_instance& I = inst[i];
    for (int64_t m = 0; m < I.num_materials; ++m) {
      double* q = &qtab[(size_t)(b->mat_off[i] + m) * 4];
      q[0] = I.materials[m].q1;
      q[1] = I.materials[m].q1ex;
      q[2] = I.materials[m].q2;
      q[3] = I.materials[m].q2ex;
    }
    dtc[i] = I.params.dt_cfl;
  }
  for (int64_t k = 0; k < NN; ++k) cin_start[k + 1] += cin_start[k];
  for (int64_t e = 0; e < NE; ++e) eie_start[e + 1] += eie_start[e];

  if (stream) {
    b->stream = static_cast<cudaStream_t>(stream);
  } else {
    CUDA_TRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    b->own_stream = true;
  }
  TRY(balloc(b, &b->d_nie, (size_t)NE * 8));
  TRY(balloc(b, &b->d_cin_start, (size_t)NN + 1));
  TRY(balloc(b, &b->d_cin, cin.size()));
  TRY(balloc(b, &b->d_eie_start, (size_t)NE + 1));
  TRY(balloc(b, &b->d_eie, eie.size()));
  TRY(balloc(b, &b->d_mat, (size_t)NE));
  TRY(balloc(b, &b->d_inst_e, (size_t)NE));
  TRY(balloc(b, &b->d_inst_n, (size_t)NN));
  TRY(balloc(b, &b->d_part_start, (size_t)n + 1));
  TRY(balloc(b, &b->d_bc, (size_t)NN));
  TRY(balloc(b, &b->d_qtab, qtab.size()));
  TRY(balloc(b, &b->d_dt_cfl, (size_t)n));
  TRY(balloc(b, &b->d_lps, (size_t)n));
  TRY(balloc(b, &b->d_node_mass, (size_t)NN));
  if (fp_mode == FIERRO_FP_FMA) TRY(balloc(b, &b->d_node_rm, (size_t)NN));
  TRY(balloc(b, &b->d_elem_mass, (size_t)NE));
  TRY(balloc(b, &b->d_gamma, (size_t)NE));
  TRY(balloc(b, &b->d_csmin, (size_t)NE));
  for (int k = 0; k < 2; ++k)
    for (int d = 0; d < 3; ++d) {
      TRY(balloc(b, &b->d_x[k][d], (size_t)NN));
      TRY(balloc(b, &b->d_v[k][d], (size_t)NN));
    }
  for (int d = 0; d < 3; ++d) TRY(balloc(b, &b->d_h[d], (size_t)NN));
  TRY(balloc(b, &b->d_den, (size_t)NE));
  TRY(balloc(b, &b->d_pres, (size_t)NE));
  TRY(balloc(b, &b->d_sspd, (size_t)NE));
  TRY(balloc(b, &b->d_vol, (size_t)NE));
  TRY(balloc(b, &b->d_div[0], (size_t)NE));
  TRY(balloc(b, &b->d_div[1], (size_t)NE));
  TRY(balloc(b, &b->d_sie[0], (size_t)NE));
  TRY(balloc(b, &b->d_sie[1], (size_t)NE));
  TRY(balloc(b, &b->d_bmat, (size_t)NE * 24));
  TRY(balloc(b, &b->d_force, (size_t)NE * 24));
  TRY(balloc(b, &b->d_cfl, (size_t)(NE / kMinBatchBlock)));  // one partial per tile of the smallest block
  TRY(balloc(b, &b->d_ctrl, (size_t)n));
  TRY(balloc(b, &b->d_sync, 3));
  CUDA_TRY(cudaMemsetAsync(b->d_sync, 0, 3 * sizeof(unsigned int), b->stream));
  TRY(put(b, b->d_nie, nie));
  TRY(put(b, b->d_cin_start, cin_start));
  TRY(put(b, b->d_cin, cin));
  TRY(put(b, b->d_eie_start, eie_start));
  TRY(put(b, b->d_eie, eie));
  TRY(put(b, b->d_mat, mat));
  TRY(put(b, b->d_inst_e, inst_e));
  TRY(put(b, b->d_inst_n, inst_n));
  TRY(put(b, b->d_part_start, b->part_start));
  TRY(put(b, b->d_bc, bc));
  TRY(put(b, b->d_qtab, qtab));
  TRY(put(b, b->d_dt_cfl, dtc));
  TRY(put(b, b->d_lps, b->lps));
  // padding elements stay inert, but keep every array defined
  for (double* p : {b->d_elem_mass, b->d_gamma, b->d_csmin, b->d_den, b->d_pres, b->d_sspd, b->d_vol, b->d_div[0],
                    b->d_div[1], b->d_sie[0], b->d_sie[1]})
    CUDA_TRY(cudaMemsetAsync(p, 0, sizeof(double) * (size_t)NE, b->stream));
  CUDA_TRY(cudaMemsetAsync(b->d_force, 0, sizeof(double) * (size_t)NE * 24, b->stream));
  CUDA_TRY(cudaMemsetAsync(b->d_bmat, 0, sizeof(double) * (size_t)NE * 24, b->stream));
  CUDA_TRY(cudaMemsetAsync(b->d_ctrl, 0, sizeof(Ctrl) * (size_t)n, b->stream));
  size_t stage = 0;
  for (int64_t i = 0; i < n; ++i)
    stage = std::max<size_t>(stage, (size_t)std::max(inst[i].mesh.num_nodes, inst[i].mesh.num_elems));
  b->stage_elems = stage;
  CUDA_TRY(cudaHostAlloc((void**)&b->h_stage, sizeof(double) * stage, cudaHostAllocDefault));
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev));
  TRY(apply_shape(b, b->shape));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return FIERRO_OK;
}

int read_ctrl(fierro_batch* b, int64_t i, Ctrl* c) {
  CUDA_TRY(cudaMemcpyAsync(c, b->d_ctrl + i, sizeof(Ctrl), cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return FIERRO_OK;
}

}  // namespace

extern "C" int fierro_batch_destroy(fierro_batch* b) {
  if (!b) return FIERRO_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (int c = 0; c < 2; ++c)
    if (b->graph[c]) cudaGraphExecDestroy(b->graph[c]);
  for (void* p : b->allocations) cudaFree(p);
  if (b->h_stage) cudaFreeHost(b->h_stage);
  if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return FIERRO_OK;
}

extern "C" int fierro_batch_create(const fierro_batch_instance* instances, int64_t num_instances, int fp_mode,
                                   void* stream, fierro_batch** out) {
  clear_error();
  NvtxRange nvtx_("fierro_batch_create");
  if (!out) return set_error(FIERRO_EINVAL, "out is NULL");
  *out = nullptr;
  fierro_batch* b = new (std::nothrow) fierro_batch();
  if (!b) return set_error(FIERRO_ENOMEM, "host allocation failed");
  int rc = create_impl(b, instances, num_instances, fp_mode, stream);
  if (rc) {
    std::string msg = fierro_last_error();
    fierro_batch_destroy(b);
    set_error(rc, "%s", msg.c_str());
    return rc;
  }
  *out = b;
  return FIERRO_OK;
}

extern "C" int fierro_batch_set_state(fierro_batch* b, int64_t i, const fierro_sgh_state* s) {
  clear_error();
  if (!b || i < 0 || i >= b->n) return set_error(FIERRO_EINVAL, "batch: bad instance index");
  if (b->started) return set_error(FIERRO_EINVAL, "batch: states are fixed once the batch has run");
  if (!s || !s->node_coords || !s->node_vel || !s->node_mass || !s->elem_den || !s->elem_pres || !s->elem_sspd ||
      !s->elem_sie || !s->elem_vol || !s->elem_mass || !s->elem_mat_id || !s->elem_statev || s->num_state_vars < 2)
    return set_error(FIERRO_EINVAL, "batch: instance %lld: required state arrays missing", (long long)i);
  const HostTopo& t = b->topo[i];
  const int64_t nn = t.nn, ne = t.ne, nsv = s->num_state_vars;
  const int64_t nmat = b->mat_off[i + 1] - b->mat_off[i];
  if (s->elem_stress)
    for (int64_t k = 0; k < ne * 18; ++k)
      if (s->elem_stress[k] != 0.0) return set_error(FIERRO_ENOTSUP, "batch: non-zero stress needs a strength model");
  for (int64_t e = 0; e < ne; ++e) {
    if (s->elem_mat_id[e] >= (uint64_t)nmat) return set_error(FIERRO_EINVAL, "batch: material id out of range");
    if (!(s->elem_vol[e] > 0.0) || !std::isfinite(s->elem_vol[e]))
      return set_error(FIERRO_ENUMERIC, "batch: instance %lld element %lld volume %g", (long long)i, (long long)e,
                       s->elem_vol[e]);
    if (!(s->elem_mass[e] > 0.0)) return set_error(FIERRO_EINVAL, "batch: element mass <= 0");
  }
  for (int64_t k = 0; k < nn; ++k)
    if (!(s->node_mass[k] > 0.0)) return set_error(FIERRO_EINVAL, "batch: node mass <= 0");
  const int64_t no = b->node_off[i], eo = b->elem_off[i];
  for (int rb = 0; rb < 2; ++rb) {
    const int bin = rb ^ 1;
    for (int d = 0; d < 3; ++d) {
      TRY(gather_up(b, b->d_x[bin][d], no, s->node_coords + (size_t)rb * nn * 3, t.node_int2ext, 3, d));
      TRY(gather_up(b, b->d_v[bin][d], no, s->node_vel + (size_t)rb * nn * 3, t.node_int2ext, 3, d));
    }
    TRY(gather_up(b, b->d_sie[bin], eo, s->elem_sie + (size_t)rb * ne, t.elem_int2ext, 1, 0));
  }
  TRY(gather_up(b, b->d_node_mass, no, s->node_mass, t.node_int2ext, 1, 0));
  TRY(gather_up(b, b->d_den, eo, s->elem_den, t.elem_int2ext, 1, 0));
  TRY(gather_up(b, b->d_pres, eo, s->elem_pres, t.elem_int2ext, 1, 0));
  TRY(gather_up(b, b->d_sspd, eo, s->elem_sspd, t.elem_int2ext, 1, 0));
  TRY(gather_up(b, b->d_vol, eo, s->elem_vol, t.elem_int2ext, 1, 0));
  TRY(gather_up(b, b->d_elem_mass, eo, s->elem_mass, t.elem_int2ext, 1, 0));
  TRY(gather_up(b, b->d_gamma, eo, s->elem_statev, t.elem_int2ext, (size_t)nsv, 0));
  TRY(gather_up(b, b->d_csmin, eo, s->elem_statev, t.elem_int2ext, (size_t)nsv, 1));
  if (s->elem_div) TRY(gather_up(b, b->d_div[1], eo, s->elem_div, t.elem_int2ext, 1, 0));
  std::vector<int32_t> mat((size_t)ne);
  for (int64_t e = 0; e < ne; ++e) mat[e] = (int32_t)(s->elem_mat_id[t.elem_int2ext[e]] + (uint64_t)b->mat_off[i]);
  CUDA_TRY(cudaMemcpyAsync(b->d_mat + eo, mat.data(), sizeof(int32_t) * (size_t)ne, cudaMemcpyHostToDevice, b->stream));
  Ctrl c{};
  c.dt = b->dt_start[i];
  c.time_value = 0.0;
  c.graphics_time = b->lps[i].graphics_dt_ival;
  CUDA_TRY(cudaMemcpyAsync(b->d_ctrl + i, &c, sizeof(Ctrl), cudaMemcpyHostToDevice, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  b->has_state[i] = 1;
  return FIERRO_OK;
}

extern "C" int fierro_batch_run(fierro_batch* b, int64_t cycles) {
  clear_error();
  NvtxRange nvtx_("fierro_batch_run");
  if (!b) return set_error(FIERRO_EINVAL, "batch is NULL");
  if (!b->started) {
    for (int64_t i = 0; i < b->n; ++i)
      if (!b->has_state[i]) return set_error(FIERRO_EINVAL, "batch: instance %lld has no state", (long long)i);
    // prime every instance: corner normals, divergence and CFL partials
    if (b->d_node_rm) b->ks->reciprocal(b->d_node_mass, b->d_node_rm, (int)b->NN, b->stream);
    b->ks->elem(b_elem(b, 0, 0, 1.0, 0), 2, b->stream);
    CUDA_TRY(cudaGetLastError());
    b->started = true;
  }
  for (int64_t k = 0; k < cycles; ++k) {
    CUDA_TRY(cudaGraphLaunch(b->graph[b->enq_cycles & 1], b->stream));
    b->enq_cycles++;
  }
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  TRY(check_sync(b));
  std::vector<Ctrl> cs((size_t)b->n);
  CUDA_TRY(cudaMemcpy(cs.data(), b->d_ctrl, sizeof(Ctrl) * (size_t)b->n, cudaMemcpyDeviceToHost));
  for (int64_t i = 0; i < b->n; ++i) {
    if (cs[i].status & FIERRO_STATUS_BAD_VOLUME)
      return set_error(FIERRO_ENUMERIC, "batch: instance %lld: non-positive element volume at cycle %lld", (long long)i,
                       cs[i].cycle);
    if (cs[i].status & FIERRO_STATUS_BAD_STATE)
      return set_error(FIERRO_ENUMERIC, "batch: instance %lld: non-finite state at cycle %lld", (long long)i,
                       cs[i].cycle);
  }
  return FIERRO_OK;
}

extern "C" int fierro_batch_get_state(fierro_batch* b, int64_t i, fierro_sgh_state* s) {
  clear_error();
  if (!b || i < 0 || i >= b->n || !s) return set_error(FIERRO_EINVAL, "batch: bad instance index or state");
  if (!b->has_state[i]) return set_error(FIERRO_EINVAL, "batch: instance %lld has no state", (long long)i);
  Ctrl c;
  TRY(read_ctrl(b, i, &c));
  const int b1 = (int)(c.cycle & 1), b0 = b1 ^ 1;
  const HostTopo& t = b->topo[i];
  const int64_t nn = t.nn, ne = t.ne, no = b->node_off[i], eo = b->elem_off[i];
  const int bins[2] = {b0, b1};
  for (int rb = 0; rb < 2; ++rb)
    for (int d = 0; d < 3; ++d) {
      if (s->node_coords)
        TRY(scatter_down(b, s->node_coords + (size_t)rb * nn * 3, b->d_x[bins[rb]][d], no, t.node_int2ext, 3, d));
      if (s->node_vel)
        TRY(scatter_down(b, s->node_vel + (size_t)rb * nn * 3, b->d_v[bins[rb]][d], no, t.node_int2ext, 3, d));
    }
  if (s->elem_sie)
    for (int rb = 0; rb < 2; ++rb)
      TRY(scatter_down(b, s->elem_sie + (size_t)rb * ne, b->d_sie[bins[rb]], eo, t.elem_int2ext, 1, 0));
  if (s->node_mass) TRY(scatter_down(b, s->node_mass, b->d_node_mass, no, t.node_int2ext, 1, 0));
  if (s->elem_den) TRY(scatter_down(b, s->elem_den, b->d_den, eo, t.elem_int2ext, 1, 0));
  if (s->elem_pres) TRY(scatter_down(b, s->elem_pres, b->d_pres, eo, t.elem_int2ext, 1, 0));
  if (s->elem_sspd) TRY(scatter_down(b, s->elem_sspd, b->d_sspd, eo, t.elem_int2ext, 1, 0));
  if (s->elem_vol) TRY(scatter_down(b, s->elem_vol, b->d_vol, eo, t.elem_int2ext, 1, 0));
  if (s->elem_mass) TRY(scatter_down(b, s->elem_mass, b->d_elem_mass, eo, t.elem_int2ext, 1, 0));
  if (s->elem_div) {
    const long long stages_done = c.cycle * b->rk_num_stages;
    const int qb = stages_done == 0 ? 1 : (int)((stages_done - 1) & 1);
    TRY(scatter_down(b, s->elem_div, b->d_div[qb], eo, t.elem_int2ext, 1, 0));
  }
  if (s->elem_stress) std::memset(s->elem_stress, 0, sizeof(double) * (size_t)ne * 18);
  if (s->corner_force)
    for (int r = 0; r < 24; ++r)
      TRY(scatter_down(b, s->corner_force, b->d_force + (size_t)r * b->NE, eo, t.elem_int2ext, 24, (size_t)r));
  return FIERRO_OK;
}

extern "C" int fierro_batch_set_shape(fierro_batch* b, const fierro_batch_shape* shape) {
  clear_error();
  if (!b || !shape) return set_error(FIERRO_EINVAL, "batch or shape is NULL");
  if (b->started) return set_error(FIERRO_EINVAL, "batch: the launch shape is fixed once the batch has run");
  return apply_shape(b, *shape);
}

extern "C" int fierro_batch_get_shape(const fierro_batch* b, fierro_batch_shape* shape) {
  clear_error();
  if (!b || !shape) return set_error(FIERRO_EINVAL, "batch or shape is NULL");
  *shape = b->shape;
  return FIERRO_OK;
}

namespace {

// The cycle-mutable device arrays of a batch (everything a cycle writes except
// the CFL partials, which the priming pass rewrites), for the autotuner's
// save / restore around each timed candidate.
std::vector<std::pair<void*, size_t>> mutable_arrays(fierro_batch* b) {
  const size_t nn = sizeof(double) * (size_t)b->NN, ne = sizeof(double) * (size_t)b->NE;
  std::vector<std::pair<void*, size_t>> v;
  for (int k = 0; k < 2; ++k)
    for (int d = 0; d < 3; ++d) {
      v.push_back({b->d_x[k][d], nn});
      v.push_back({b->d_v[k][d], nn});
    }
  for (int d = 0; d < 3; ++d) v.push_back({b->d_h[d], nn});
  for (double* p : {b->d_sie[0], b->d_sie[1], b->d_den, b->d_pres, b->d_sspd, b->d_vol, b->d_div[0], b->d_div[1]})
    v.push_back({p, ne});
  v.push_back({b->d_bmat, 24 * ne});
  v.push_back({b->d_force, 24 * ne});
  v.push_back({b->d_ctrl, sizeof(Ctrl) * (size_t)b->n});
  return v;
}

int copy_arrays(fierro_batch* b, char* save, const std::vector<std::pair<void*, size_t>>& arrs, bool to_save) {
  size_t off = 0;
  for (const auto& a : arrs) {
    CUDA_TRY(cudaMemcpyAsync(to_save ? save + off : a.first, to_save ? a.first : save + off, a.second,
                             cudaMemcpyDeviceToDevice, b->stream));
    off += a.second;
  }
  return FIERRO_OK;
}

// Primes the uploaded state with the current shape, runs `warm` cycles, then
// times `cycles` cycles of the captured graphs; ms per cycle.
int time_shape(fierro_batch* b, int warm, int cycles, double* ms) {
  if (b->d_node_rm) b->ks->reciprocal(b->d_node_mass, b->d_node_rm, (int)b->NN, b->stream);
  b->ks->elem(b_elem(b, 0, 0, 1.0, 0), 2, b->stream);
  CUDA_TRY(cudaGetLastError());
  long long k = 0;
  for (; k < warm; ++k) CUDA_TRY(cudaGraphLaunch(b->graph[k & 1], b->stream));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  cudaError_t err = cudaEventRecord(e0, b->stream);
  for (long long i = 0; i < cycles && err == cudaSuccess; ++i, ++k) err = cudaGraphLaunch(b->graph[k & 1], b->stream);
  if (err == cudaSuccess) err = cudaEventRecord(e1, b->stream);
  if (err == cudaSuccess) err = cudaEventSynchronize(e1);
  float t = 0.0f;
  if (err == cudaSuccess) err = cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (err != cudaSuccess) return set_error(FIERRO_ECUDA, "batch autotune: %s", cudaGetErrorString(err));
  TRY(check_sync(b));
  *ms = (double)t / std::max(cycles, 1);
  return FIERRO_OK;
}

}  // namespace

extern "C" int fierro_batch_autotune(fierro_batch* b, int64_t cycles, fierro_batch_shape* chosen) {
  clear_error();
  NvtxRange nvtx_("fierro_batch_autotune");
  if (!b) return set_error(FIERRO_EINVAL, "batch is NULL");
  if (b->started) return set_error(FIERRO_EINVAL, "batch: autotune before the first fierro_batch_run");
  if (cycles < 1 || cycles > 1000) return set_error(FIERRO_EINVAL, "batch autotune: cycles must be 1..1000");
  for (int64_t i = 0; i < b->n; ++i)
    if (!b->has_state[i]) return set_error(FIERRO_EINVAL, "batch: instance %lld has no state", (long long)i);
  const auto arrs = mutable_arrays(b);
  size_t total = 0;
  for (const auto& a : arrs) total += a.second;
  char* save = nullptr;
  CUDA_TRY(cudaMalloc(&save, total));
  b->tune_shapes.clear();
  b->tune_ms.clear();
  int rc = copy_arrays(b, save, arrs, true);
  const fierro_batch_shape start = b->shape;
  fierro_batch_shape best = b->shape;
  double best_ms = 0.0;
  bool have = false;
  // coordinate descent: force block, node block, element block, persistent grid
  auto trial = [&](fierro_batch_shape sh) -> int {
    for (size_t i = 0; i < b->tune_shapes.size(); ++i) {
      const fierro_batch_shape& o = b->tune_shapes[i];
      if (o.force_block == sh.force_block && o.node_block == sh.node_block && o.elem_block == sh.elem_block &&
          o.persistent == sh.persistent && o.fused_stage == sh.fused_stage)
        return FIERRO_OK;
    }
    TRY(copy_arrays(b, save, arrs, false));
    TRY(apply_shape(b, sh));
    double ms = 0.0;
    TRY(time_shape(b, 1, (int)cycles, &ms));
    b->tune_shapes.push_back(sh);
    b->tune_ms.push_back(ms);
    if (!have || ms < best_ms) {
      best = sh;
      best_ms = ms;
      have = true;
    }
    return FIERRO_OK;
  };
  const int force_blocks[] = {128, 64, 32}, node_blocks[] = {256, 128, 512, 64}, elem_blocks[] = {128, 64, 32};
  const int persist[] = {0, 1, 2};
  for (int fb : force_blocks) {
    if (rc) break;
    fierro_batch_shape sh = best;
    sh.force_block = fb;
    rc = trial(sh);
  }
  for (int nb : node_blocks) {
    if (rc) break;
    fierro_batch_shape sh = best;
    sh.node_block = nb;
    rc = trial(sh);
  }
  for (int eb : elem_blocks) {
    if (rc) break;
    fierro_batch_shape sh = best;
    sh.elem_block = eb;
    rc = trial(sh);
  }
  for (int p : persist) {
    if (rc) break;
    fierro_batch_shape sh = best;
    sh.persistent = p;
    rc = trial(sh);
  }
  // the fused stage (one cooperative launch per stage, at the chosen element
  // block); a candidate the device cannot run is left out of the choice
  if (!rc) {
    fierro_batch_shape sh = best;
    sh.persistent = 0;
    sh.fused_stage = 1;
    if (trial(sh) != FIERRO_OK) clear_error();
  }
  // the uploaded state back (also after a failed candidate), with the chosen
  // shape, or the shape the batch had when the tuning failed
  const int rc_restore = copy_arrays(b, save, arrs, false);
  cudaStreamSynchronize(b->stream);
  cudaFree(save);
  if (rc) {
    apply_shape(b, start);
    return rc;
  }
  if (rc_restore) return rc_restore;
  TRY(apply_shape(b, best));
  if (chosen) *chosen = best;
  return FIERRO_OK;
}

extern "C" int fierro_batch_tune_log(const fierro_batch* b, fierro_batch_shape* shapes, double* ms_per_cycle,
                                     int64_t capacity, int64_t* count) {
  clear_error();
  if (!b || !count) return set_error(FIERRO_EINVAL, "batch or count is NULL");
  const int64_t n = (int64_t)b->tune_shapes.size();
  *count = n;
  for (int64_t i = 0; i < n && i < capacity; ++i) {
    if (shapes) shapes[i] = b->tune_shapes[(size_t)i];
    if (ms_per_cycle) ms_per_cycle[i] = b->tune_ms[(size_t)i];
  }
  return FIERRO_OK;
}

extern "C" int fierro_batch_time(fierro_batch* b, int64_t i, double* time_value, double* dt, int64_t* cycle) {
  clear_error();
  if (!b || i < 0 || i >= b->n) return set_error(FIERRO_EINVAL, "batch: bad instance index");
  Ctrl c;
  TRY(read_ctrl(b, i, &c));
  if (time_value) *time_value = c.time_value;
  if (dt) *dt = c.dt;
  if (cycle) *cycle = c.cycle;
  return FIERRO_OK;
}

extern "C" int64_t fierro_batch_num_instances(const fierro_batch* b) { return b ? b->n : 0; }
extern "C" int64_t fierro_batch_device_bytes(const fierro_batch* b) { return b ? (int64_t)b->dev_bytes : 0; }
