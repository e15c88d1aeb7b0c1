// C ABI of libfierro_sgh: the persistent handle (device-resident mesh and state,
// per-parity CUDA graphs of one cycle) and the one-shot fierro_sgh_solve.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <unistd.h>

#include <cuda_runtime.h>

#include "sgh_handle.h"
#include "sgh_rz.h"
#include "sgh_topo.h"
#include "sgh_user_mat.cuh"

using namespace fierro;

namespace fierro {
namespace hd {

int upload_raw(fierro_sgh* h, void* dst, const void* src, size_t bytes) {
  CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  return FIERRO_OK;
}

// Permuted upload through the pinned double buffer: dst[i] = src[map[i]*stride + off].
int upload_gather(fierro_sgh* h, double* dst, const double* src, const std::vector<int64_t>& map,
                  size_t stride, size_t off, int* slot) {
  const int64_t n = (int64_t)map.size();
  double* st = h->h_stage[*slot];
  CUDA_TRY(cudaEventSynchronize(h->stage_ev[*slot]));
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) st[i] = src[(size_t)map[i] * stride + off];
  CUDA_TRY(cudaMemcpyAsync(dst, st, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(cudaEventRecord(h->stage_ev[*slot], h->stream));
  *slot ^= 1;
  return FIERRO_OK;
}

// Permuted download: out[map[i]*stride + off] = src[i].
int download_scatter(fierro_sgh* h, double* out, const double* src, const std::vector<int64_t>& map,
                     size_t stride, size_t off) {
  const int64_t n = (int64_t)map.size();
  double* st = h->h_stage[0];
  CUDA_TRY(cudaMemcpyAsync(st, src, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) out[(size_t)map[i] * stride + off] = st[i];
  return FIERRO_OK;
}

int check_status(fierro_sgh* h) {
  Ctrl c;
  CUDA_TRY(cudaMemcpyAsync(&c, h->d_ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (c.status & FIERRO_STATUS_BAD_VOLUME)
    return set_error(FIERRO_ENUMERIC, "non-positive or non-finite element volume at cycle %lld", c.cycle);
  if (c.status & FIERRO_STATUS_BAD_STATE)
    return set_error(FIERRO_ENUMERIC, "non-finite energy or pressure at cycle %lld", c.cycle);
  return FIERRO_OK;
}

ForceArgs force_args(fierro_sgh* h, int rb, int q) {
  ForceArgs a{};
  a.ne = (int)h->ne;
  a.nie = h->d_nie;
  a.eie_start = h->d_eie_start;
  a.eie = h->d_eie;
  a.mat = h->d_mat;
  a.qtab = h->d_qtab;
  a.bmat = h->d_bmat;
  a.u = h->d_v[rb][0];
  a.v = h->d_v[rb][1];
  a.w = h->d_v[rb][2];
  a.den = h->d_den;
  a.pres = h->d_pres;
  a.sspd = h->d_sspd;
  a.vol = h->d_vol;
  a.div = h->d_div[q];
  a.force = h->d_force;
  a.ctrl = h->d_ctrl;
  a.fuzz = h->lp.fuzz;
  a.small = h->lp.small;
  a.block = h->blk_force;
  return a;
}

NodeArgs node_args(fierro_sgh* h, int c, double alpha) {
  NodeArgs a{};
  a.nn = (int)h->nn;
  a.ne = (int)h->ne;
  a.cin_start = h->d_cin_start;
  a.cin = h->d_cin;
  a.force = h->d_force;
  a.node_mass = h->d_node_mass;
  a.node_rm = h->d_node_rm;
  a.bc_mask = h->d_bc;
  a.u0 = h->d_v[c][0];
  a.v0 = h->d_v[c][1];
  a.w0 = h->d_v[c][2];
  a.x0 = h->d_x[c][0];
  a.y0 = h->d_x[c][1];
  a.z0 = h->d_x[c][2];
  a.u1 = h->d_v[c ^ 1][0];
  a.v1 = h->d_v[c ^ 1][1];
  a.w1 = h->d_v[c ^ 1][2];
  a.x1 = h->d_x[c ^ 1][0];
  a.y1 = h->d_x[c ^ 1][1];
  a.z1 = h->d_x[c ^ 1][2];
  a.hx = h->d_h[0];
  a.hy = h->d_h[1];
  a.hz = h->d_h[2];
  a.ctrl = h->d_ctrl;
  a.rk_alpha = alpha;
  a.block = h->blk_node;
  return a;
}

ElemArgs elem_args(fierro_sgh* h, int cur_bin, int c, double alpha, int div_out) {
  ElemArgs a{};
  a.ne = (int)h->ne;
  a.nie = h->d_nie;
  a.x = h->d_x[cur_bin][0];
  a.y = h->d_x[cur_bin][1];
  a.z = h->d_x[cur_bin][2];
  a.u = h->d_v[cur_bin][0];
  a.v = h->d_v[cur_bin][1];
  a.w = h->d_v[cur_bin][2];
  a.hx = h->d_h[0];
  a.hy = h->d_h[1];
  a.hz = h->d_h[2];
  a.force = h->d_force;
  a.mass = h->d_elem_mass;
  a.sie0 = h->d_sie[c];
  a.sie1 = h->d_sie[c ^ 1];
  a.gamma = h->d_gamma;
  a.csmin = h->d_csmin;
  a.den = h->d_den;
  a.pres = h->d_pres;
  a.sspd = h->d_sspd;
  a.vol = h->d_vol;
  a.div = h->d_div[div_out];
  a.bmat = h->d_bmat;
  a.cfl_part = h->d_cfl;
  a.ctrl = h->d_ctrl;
  a.rk_alpha = alpha;
  a.dt_cfl = h->lp.dt_cfl;
  a.fuzz = h->lp.fuzz;
  a.block = h->blk_elem;
  return a;
}

ForceArgs stage_force_args(fierro_sgh* h, int c, int s) {
  const int rb = (s == 0) ? c : (c ^ 1);
  ForceArgs a = force_args(h, rb, div_parity(h, c, s));
  if (h->strength) {
    // stress(1) is the cycle-start bin until the first stage writes bin c^1
    a.stress_cur = h->d_stress[rb];
    a.stress0 = h->d_stress[c];
    a.stress_out = h->d_stress[c ^ 1];
    a.stype = h->d_stype;
    a.statev = h->d_statev;
    a.sie0 = h->d_sie[c];
    a.rk_alpha = stage_alpha(h, s);
    a.copy_stress = s == 0;
  }
  return a;
}

ElemArgs stage_elem_args(fierro_sgh* h, int c, int s) {
  ElemArgs a = elem_args(h, c ^ 1, c, stage_alpha(h, s), div_parity(h, c, s) ^ 1);
  if (h->has_hyper) {
    a.mat = h->d_mat;
    a.stype = h->d_stype;
    a.stress0 = h->d_stress[c];
    a.stress1 = h->d_stress[c ^ 1];
    a.statev = h->d_statev;
  }
  return a;
}

int cycles_done(fierro_sgh* h, long long* cyc) {
  Ctrl c;
  CUDA_TRY(cudaMemcpyAsync(&c, h->d_ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  *cyc = c.cycle;
  return FIERRO_OK;
}

}  // namespace hd
}  // namespace fierro

using namespace fierro::hd;

namespace {

// Stage s of a cycle whose start state is in bin c; with `ev`, an event is
// recorded after each launch.
int enqueue_stage_ev(fierro_sgh* h, int c, int s, cudaEvent_t* ev, size_t* k) {
  if (h->dims == 2) return rz::enqueue_stage(h, c, s, ev, k);
  h->ks->force(stage_force_args(h, c, s), h->stream);
  if (ev) CUDA_TRY(cudaEventRecord(ev[(*k)++], h->stream));
  h->ks->node(node_args(h, c, stage_alpha(h, s)), h->stream);
  if (ev) CUDA_TRY(cudaEventRecord(ev[(*k)++], h->stream));
  h->ks->elem(stage_elem_args(h, c, s), (s == h->rk_num_stages - 1) ? 1 : 0, h->stream);
  if (ev) CUDA_TRY(cudaEventRecord(ev[(*k)++], h->stream));
  return FIERRO_OK;
}

void enqueue_stage(fierro_sgh* h, int c, int s) { enqueue_stage_ev(h, c, s, nullptr, nullptr); }

void enqueue_dt(fierro_sgh* h) {
  DtArgs d{};
  d.cfl_part = h->d_cfl;
  d.nparts = h->ncfl;
  d.ctrl = h->d_ctrl;
  d.lp = h->lp;
  h->ks->dt(d, h->stream);
}

void enqueue_cycle(fierro_sgh* h, int c) {
  enqueue_dt(h);
  for (int s = 0; s < h->rk_num_stages; ++s) enqueue_stage(h, c, s);
  h->ks->end(h->d_ctrl, h->lp, h->stream);
  // a write event of this cycle: snapshot of the state it left in bin c ^ 1
  if (h->out) xfer::launch_snapshot(output_snap_args(h, c ^ 1, 0), h->stream);
}

int build_graphs(fierro_sgh* h) {
  for (int c = 0; c < 2; ++c) {
    if (h->graph[c]) {
      cudaGraphExecDestroy(h->graph[c]);
      h->graph[c] = nullptr;
    }
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    enqueue_cycle(h, c);
    CUDA_TRY(cudaStreamEndCapture(h->stream, &g));
    cudaError_t err = cudaGraphInstantiate(&h->graph[c], g, 0);
    cudaGraphDestroy(g);
    if (err != cudaSuccess) return set_error(FIERRO_ECUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(err));
  }
  return FIERRO_OK;
}

}  // namespace

int fierro::rebuild_graphs(fierro_sgh* h) {
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  return build_graphs(h);
}

namespace {

int validate_params(const fierro_sgh_params* p) {
  if (!p) return set_error(FIERRO_EINVAL, "params is NULL");
  if (p->rk_num_stages < 1 || p->rk_num_stages > 8)
    return set_error(FIERRO_EINVAL, "rk_num_stages %lld out of range 1..8", (long long)p->rk_num_stages);
  if (p->graphics_cyc_ival < 1) return set_error(FIERRO_EINVAL, "graphics_cyc_ival must be >= 1");
  if (!(p->dt_cfl > 0) || !(p->dt_max > 0) || !(p->dt_min > 0) || !(p->dt_start > 0))
    return set_error(FIERRO_EINVAL, "dt_cfl, dt_max, dt_min and dt_start must be positive");
  return FIERRO_OK;
}

}  // namespace

extern "C" int fierro_sgh_destroy(fierro_sgh* h) {
  if (!h) return FIERRO_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  output_release(h);
  adj_release(h);
  adj_branches_release(h);
  for (int c = 0; c < 2; ++c)
    if (h->graph[c]) cudaGraphExecDestroy(h->graph[c]);
  for (void* p : h->allocations) cudaFree(p);
  if (h->d_statev) cudaFree(h->d_statev);
  for (int i = 0; i < 2; ++i) {
    if (h->h_stage[i]) cudaFreeHost(h->h_stage[i]);
    if (h->stage_ev[i]) cudaEventDestroy(h->stage_ev[i]);
  }
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return FIERRO_OK;
}

static int create_impl(fierro_sgh* h, const fierro_mesh* mesh, const fierro_material* materials,
                       int64_t num_materials, const fierro_boundary* boundaries, int64_t num_bcs,
                       const fierro_sgh_params* params, int fp_mode, void* stream) {
  TRY(validate_params(params));
  if (fp_mode != FIERRO_FP_EXACT && fp_mode != FIERRO_FP_FMA)
    return set_error(FIERRO_EINVAL, "fp_mode %d unknown", fp_mode);
  if (num_materials < 1 || !materials) return set_error(FIERRO_EINVAL, "need at least one material");
  TRY(check_mesh_header(mesh));
  h->dims = mesh_dims(mesh);
  {
    const char* env = std::getenv("FIERRO_FAIL_ALLOC_AFTER");
    h->alloc_limit = env ? std::strtoll(env, nullptr, 10) : -1;
  }
  for (int64_t m = 0; m < num_materials; ++m) {
    if (materials[m].eos_model != 0) return set_error(FIERRO_ENOTSUP, "material %lld: only the ideal-gas EOS", (long long)m);
    if (materials[m].strength_type < 0 || materials[m].strength_type > 2)
      return set_error(FIERRO_EINVAL, "material %lld: strength_type %d unknown (0 none, 1 hypo, 2 hyper)",
                       (long long)m, materials[m].strength_type);
    if (materials[m].strength_type != 0) h->strength = true;
    if (materials[m].strength_type == 2) h->has_hyper = true;
  }
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  TRY(h->dims == 2 ? validate_bcs_rz(boundaries, num_bcs) : validate_bcs(boundaries, num_bcs));
  if (h->dims == 2) {
    h->nn = mesh->num_nodes;
    h->ne = mesh->num_elems;
    h->nmat = (int)num_materials;
    h->fp_mode = fp_mode;
    h->ks = (fp_mode == FIERRO_FP_EXACT) ? &kernels_exact() : &kernels_fma();
    h->lp = LoopParams{params->time_final, params->dt_max,  params->dt_min, params->dt_cfl,
                       params->graphics_dt_ival, params->fuzz, params->small, params->graphics_cyc_ival};
    h->rk_num_stages = (int)params->rk_num_stages;
    h->dt_start = params->dt_start;
    h->tiny = params->tiny;
    if (stream) {
      h->stream = static_cast<cudaStream_t>(stream);
    } else {
      CUDA_TRY(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
      h->own_stream = true;
    }
    TRY(rz::create(h, mesh, materials, num_materials, boundaries, num_bcs));
    TRY(build_graphs(h));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return FIERRO_OK;
  }
  {
    const char* env = std::getenv("FIERRO_STAGED_TRANSFERS");
    h->direct_host = xfer::direct_host_access() && !(env && env[0] == '1');
  }
  // with direct host access the GPU builds the topology from the caller's arrays
  // (sgh_topo.cu); otherwise the host builder does
  if (!h->direct_host) TRY(build_topology(mesh, boundaries, num_bcs, true, &h->topo));
  h->nn = mesh->num_nodes;
  h->ne = mesh->num_elems;
  h->nmat = (int)num_materials;
  h->fp_mode = fp_mode;
  h->ks = (fp_mode == FIERRO_FP_EXACT) ? &kernels_exact() : &kernels_fma();
  h->lp = LoopParams{params->time_final, params->dt_max,  params->dt_min, params->dt_cfl,
                     params->graphics_dt_ival, params->fuzz, params->small, params->graphics_cyc_ival};
  h->rk_num_stages = (int)params->rk_num_stages;
  h->dt_start = params->dt_start;
  if (stream) {
    h->stream = static_cast<cudaStream_t>(stream);
  } else {
    CUDA_TRY(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    h->own_stream = true;
  }
  const size_t nn = (size_t)h->nn, ne = (size_t)h->ne;
  const HostTopo& t = h->topo;
  TRY(dalloc(h, &h->d_nie, ne * 8));
  TRY(dalloc(h, &h->d_cin_start, nn + 1));
  TRY(dalloc(h, &h->d_cin, ne * 8));
  TRY(dalloc(h, &h->d_eie_start, ne + 1));
  if (!h->direct_host) TRY(dalloc(h, &h->d_eie, t.eie.size()));
  TRY(dalloc(h, &h->d_mat, ne));
  TRY(dalloc(h, &h->d_bc, nn));
  TRY(dalloc(h, &h->d_qtab, (size_t)num_materials * 4));
  TRY(dalloc(h, &h->d_node_mass, nn));
  if (h->fp_mode == FIERRO_FP_FMA) TRY(dalloc(h, &h->d_node_rm, nn));
  TRY(dalloc(h, &h->d_elem_mass, ne));
  TRY(dalloc(h, &h->d_gamma, ne));
  TRY(dalloc(h, &h->d_csmin, ne));
  for (int b = 0; b < 2; ++b)
    for (int d = 0; d < 3; ++d) {
      TRY(dalloc(h, &h->d_x[b][d], nn));
      TRY(dalloc(h, &h->d_v[b][d], nn));
    }
  for (int d = 0; d < 3; ++d) TRY(dalloc(h, &h->d_h[d], nn));
  TRY(dalloc(h, &h->d_den, ne));
  TRY(dalloc(h, &h->d_pres, ne));
  TRY(dalloc(h, &h->d_sspd, ne));
  TRY(dalloc(h, &h->d_vol, ne));
  TRY(dalloc(h, &h->d_div[0], ne));
  TRY(dalloc(h, &h->d_div[1], ne));
  TRY(dalloc(h, &h->d_sie[0], ne));
  TRY(dalloc(h, &h->d_sie[1], ne));
  TRY(dalloc(h, &h->d_bmat, ne * 24));
  TRY(dalloc(h, &h->d_force, ne * 24));
  if (h->strength) {
    TRY(dalloc(h, &h->d_stress[0], ne * 9));
    TRY(dalloc(h, &h->d_stress[1], ne * 9));
    TRY(dalloc(h, &h->d_stype, (size_t)num_materials));
    std::vector<int> st((size_t)num_materials);
    for (int64_t m = 0; m < num_materials; ++m) st[m] = materials[m].strength_type;
    TRY(upload_raw(h, h->d_stype, st.data(), sizeof(int) * st.size()));
  }
  h->blk_elem = small_mesh_block(ne, kElemBlock);
  h->blk_force = small_mesh_block(ne, kForceBlock);
  h->blk_node = small_mesh_block(nn, kNodeBlock);
  h->ncfl = (int)((ne + h->blk_elem - 1) / h->blk_elem);
  TRY(dalloc(h, &h->d_cfl, (size_t)h->ncfl));
  TRY(dalloc(h, &h->d_ctrl, 1));
  TRY(dalloc(h, &h->d_node_ext2int, nn));
  TRY(dalloc(h, &h->d_elem_ext2int, ne));
  TRY(dalloc(h, &h->d_node_int2ext, nn));
  TRY(dalloc(h, &h->d_elem_int2ext, ne));
  TRY(dalloc(h, &h->d_xfer, 1));
  TRY(dalloc(h, &h->d_energy_part, 2 * 512));
  TRY(dalloc(h, &h->d_energy_out, 2));
  h->stage_elems = std::max(nn, ne);
  for (int i = 0; i < 2; ++i) {
    CUDA_TRY(cudaHostAlloc((void**)&h->h_stage[i], sizeof(double) * h->stage_elems, cudaHostAllocDefault));
    CUDA_TRY(cudaEventCreateWithFlags(&h->stage_ev[i], cudaEventDisableTiming));
    CUDA_TRY(cudaEventRecord(h->stage_ev[i], h->stream));
  }
  if (h->direct_host) {
    TRY(topo::build_device(h, mesh, boundaries, num_bcs));
  } else {
    TRY(upload_raw(h, h->d_nie, t.nie.data(), sizeof(int32_t) * ne * 8));
    TRY(upload_raw(h, h->d_cin_start, t.cin_start.data(), sizeof(int32_t) * (nn + 1)));
    TRY(upload_raw(h, h->d_cin, t.cin.data(), sizeof(int32_t) * ne * 8));
    TRY(upload_raw(h, h->d_eie_start, t.eie_start.data(), sizeof(int32_t) * (ne + 1)));
    if (!t.eie.empty()) TRY(upload_raw(h, h->d_eie, t.eie.data(), sizeof(int32_t) * t.eie.size()));
    TRY(upload_raw(h, h->d_bc, t.bc_mask.data(), nn));
    h->nnz_eie = (int64_t)t.eie.size();
    std::vector<int32_t> m32(std::max(nn, ne));
    for (size_t j = 0; j < nn; ++j) m32[j] = (int32_t)t.node_ext2int[j];
    TRY(upload_raw(h, h->d_node_ext2int, m32.data(), sizeof(int32_t) * nn));
    for (size_t j = 0; j < ne; ++j) m32[j] = (int32_t)t.elem_ext2int[j];
    TRY(upload_raw(h, h->d_elem_ext2int, m32.data(), sizeof(int32_t) * ne));
    for (size_t j = 0; j < nn; ++j) m32[j] = (int32_t)t.node_int2ext[j];
    TRY(upload_raw(h, h->d_node_int2ext, m32.data(), sizeof(int32_t) * nn));
    for (size_t j = 0; j < ne; ++j) m32[j] = (int32_t)t.elem_int2ext[j];
    TRY(upload_raw(h, h->d_elem_int2ext, m32.data(), sizeof(int32_t) * ne));
  }
  std::vector<double> q((size_t)num_materials * 4);
  for (int64_t m = 0; m < num_materials; ++m) {
    q[m * 4 + 0] = materials[m].q1;
    q[m * 4 + 1] = materials[m].q1ex;
    q[m * 4 + 2] = materials[m].q2;
    q[m * 4 + 3] = materials[m].q2ex;
  }
  TRY(upload_raw(h, h->d_qtab, q.data(), sizeof(double) * q.size()));
  CUDA_TRY(cudaMemsetAsync(h->d_ctrl, 0, sizeof(Ctrl), h->stream));
  CUDA_TRY(cudaMemsetAsync(h->d_force, 0, sizeof(double) * ne * 24, h->stream));
  TRY(build_graphs(h));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  return FIERRO_OK;
}

extern "C" int fierro_sgh_create(const fierro_mesh* mesh, const fierro_material* materials, int64_t num_materials,
                                 const fierro_boundary* boundaries, int64_t num_bcs,
                                 const fierro_sgh_params* params, int fp_mode, void* stream, fierro_sgh** out) {
  clear_error();
  NvtxRange nvtx_("fierro_sgh_create");
  if (!out) return set_error(FIERRO_EINVAL, "out is NULL");
  *out = nullptr;
  fierro_sgh* h = new (std::nothrow) fierro_sgh();
  if (!h) return set_error(FIERRO_ENOMEM, "host allocation failed");
  int rc = create_impl(h, mesh, materials, num_materials, boundaries, num_bcs, params, fp_mode, stream);
  if (rc) {
    std::string msg = fierro_last_error();
    fierro_sgh_destroy(h);
    set_error(rc, "%s", msg.c_str());
    return rc;
  }
  *out = h;
  return FIERRO_OK;
}

// Loop scalars, bin bookkeeping and the priming element pass of a freshly
// uploaded state.
static int finish_set_state(fierro_sgh* h, double time_value, double graphics_time, double dt) {
  Ctrl c{};
  c.dt = dt;
  c.time_value = time_value;
  c.graphics_time = graphics_time;
  TRY(upload_raw(h, h->d_ctrl, &c, sizeof(Ctrl)));
  h->base = 0;
  h->enq_cycles = 0;
  h->stage = 0;
  if (h->d_node_rm) h->ks->reciprocal(h->d_node_mass, h->d_node_rm, (int)h->nn, h->stream);
  // prime: corner normals, divergence and CFL partials of the uploaded state
  if (h->dims == 2) TRY(rz::prime(h));
  else h->ks->elem(elem_args(h, 0, 0, 1.0, 0), 2, h->stream);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->has_state = true;
  return FIERRO_OK;
}

// The device copy of the element state variables of a strength handle, sized
// for nsv columns; the cycle graphs hold its address, so a new allocation
// re-captures them.
static int size_statev(fierro_sgh* h, int64_t nsv) {
  if (!h->strength || (h->d_statev && h->nsv == nsv)) return FIERRO_OK;
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (h->d_statev) {
    cudaFree(h->d_statev);
    h->dev_bytes -= sizeof(double) * (size_t)(h->nsv * h->ne);
    h->d_statev = nullptr;
  }
  const size_t bytes = sizeof(double) * (size_t)(nsv * h->ne);
  cudaError_t err = cudaMalloc(&h->d_statev, bytes);
  if (err != cudaSuccess) {
    h->d_statev = nullptr;
    h->nsv = 0;
    return set_error(FIERRO_ENOMEM, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(err));
  }
  h->dev_bytes += bytes;
  h->nsv = nsv;
  return build_graphs(h);
}

// The first index of a non-zero value (-1 if none), over all host threads.
static long long first_nonzero(const double* p, int64_t n) {
  long long first = -1;
#pragma omp parallel
  {
    long long mine = -1;
#pragma omp for schedule(static)
    for (int64_t i = 0; i < n; ++i)
      if (p[i] != 0.0 && mine < 0) mine = i;
#pragma omp critical
    if (mine >= 0 && (first < 0 || mine < first)) first = mine;
  }
  return first;
}

// p[0..n) = 0.0, over all host threads.
static void zero_parallel(double* p, size_t n) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) p[i] = 0.0;
}

static int set_state_impl(fierro_sgh* h, const fierro_sgh_state* s, double time_value, double graphics_time,
                          double dt) {
  if (!s || !s->node_coords || !s->node_vel || !s->node_mass || !s->elem_den || !s->elem_pres || !s->elem_sspd ||
      !s->elem_sie || !s->elem_vol || !s->elem_mass || !s->elem_mat_id || !s->elem_statev)
    return set_error(FIERRO_EINVAL, "set_state: required state arrays missing");
  if (s->num_state_vars < 2) return set_error(FIERRO_EINVAL, "set_state: need num_state_vars >= 2");
  if (h->strength && s->num_state_vars < kUserStrengthStateVars)
    return set_error(FIERRO_EINVAL, "set_state: the strength model reads %d state variables, the state has %lld",
                     kUserStrengthStateVars, (long long)s->num_state_vars);
  const int64_t nn = h->nn, ne = h->ne, nsv = s->num_state_vars;
  const HostTopo& t = h->topo;
  h->has_state = false;
  TRY(size_statev(h, nsv));
  if (h->dims == 2 && !h->direct_host) {
    TRY(rz::set_state(h, s));
    return finish_set_state(h, time_value, graphics_time, dt);
  }
  if (h->direct_host) {
    // the GPU reads the caller's arrays and validates them in the same pass
    h->has_state = false;
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    output_reset(h);
    XferStatus xs{};
    // a gas-only handle needs the caller's stress to be zero: the host checks it
    // while the GPU reads the rest of the state
    const bool host_check = s->elem_stress && !h->strength;
    fierro_sgh_state sg = *s;
    if (host_check) sg.elem_stress = nullptr;
    TRY(xfer::upload_state(h, &sg, &xs, false));
    const long long nonzero = host_check ? first_nonzero(s->elem_stress, ne * 18) : -1;
    TRY(xfer::finish_upload(h, &xs));
    if (nonzero >= 0) {
      xs.flags |= 1u << XferStatus::STRESS;
      xs.first[XferStatus::STRESS] = nonzero;
    }
    if (xs.flags & (1u << XferStatus::STRESS))
      return set_error(FIERRO_ENOTSUP, "set_state: non-zero stress (value %lld) needs a handle with a strength "
                       "material", xs.first[XferStatus::STRESS]);
    if (xs.flags & (1u << XferStatus::MAT_ID))
      return set_error(FIERRO_EINVAL, "set_state: element %lld material id out of range", xs.first[XferStatus::MAT_ID]);
    if (xs.flags & (1u << XferStatus::VOLUME))
      return set_error(FIERRO_ENUMERIC, "set_state: element %lld has a non-positive or non-finite volume",
                       xs.first[XferStatus::VOLUME]);
    if (xs.flags & (1u << XferStatus::MASS))
      return set_error(FIERRO_EINVAL, "set_state: element %lld mass <= 0", xs.first[XferStatus::MASS]);
    if (xs.flags & (1u << XferStatus::NODE_MASS))
      return set_error(FIERRO_EINVAL, "set_state: node %lld mass <= 0", xs.first[XferStatus::NODE_MASS]);
    return finish_set_state(h, time_value, graphics_time, dt);
  }
  if (s->elem_stress && !h->strength)
    for (int64_t i = 0; i < ne * 18; ++i)
      if (s->elem_stress[i] != 0.0)
        return set_error(FIERRO_ENOTSUP, "set_state: non-zero stress needs a handle with a strength material");
  for (int64_t e = 0; e < ne; ++e) {
    if (s->elem_mat_id[e] >= (uint64_t)h->nmat)
      return set_error(FIERRO_EINVAL, "set_state: element %lld material id out of range", (long long)e);
    if (!(s->elem_vol[e] > 0.0) || !std::isfinite(s->elem_vol[e]))
      return set_error(FIERRO_ENUMERIC, "set_state: element %lld has volume %g", (long long)e, s->elem_vol[e]);
    if (!(s->elem_mass[e] > 0.0)) return set_error(FIERRO_EINVAL, "set_state: element %lld mass <= 0", (long long)e);
  }
  for (int64_t n = 0; n < nn; ++n)
    if (!(s->node_mass[n] > 0.0)) return set_error(FIERRO_EINVAL, "set_state: node %lld mass <= 0", (long long)n);
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  output_reset(h);
  int slot = 0;
  // reference bin 1 -> device bin 0 (current), bin 0 -> device bin 1
  for (int rb = 0; rb < 2; ++rb) {
    const int b = rb ^ 1;
    for (int d = 0; d < 3; ++d) {
      TRY(upload_gather(h, h->d_x[b][d], s->node_coords + (size_t)rb * nn * 3, t.node_int2ext, 3, d, &slot));
      TRY(upload_gather(h, h->d_v[b][d], s->node_vel + (size_t)rb * nn * 3, t.node_int2ext, 3, d, &slot));
    }
    TRY(upload_gather(h, h->d_sie[b], s->elem_sie + (size_t)rb * ne, t.elem_int2ext, 1, 0, &slot));
  }
  TRY(upload_gather(h, h->d_node_mass, s->node_mass, t.node_int2ext, 1, 0, &slot));
  TRY(upload_gather(h, h->d_den, s->elem_den, t.elem_int2ext, 1, 0, &slot));
  TRY(upload_gather(h, h->d_pres, s->elem_pres, t.elem_int2ext, 1, 0, &slot));
  TRY(upload_gather(h, h->d_sspd, s->elem_sspd, t.elem_int2ext, 1, 0, &slot));
  TRY(upload_gather(h, h->d_vol, s->elem_vol, t.elem_int2ext, 1, 0, &slot));
  TRY(upload_gather(h, h->d_elem_mass, s->elem_mass, t.elem_int2ext, 1, 0, &slot));
  TRY(upload_gather(h, h->d_gamma, s->elem_statev, t.elem_int2ext, (size_t)nsv, 0, &slot));
  TRY(upload_gather(h, h->d_csmin, s->elem_statev, t.elem_int2ext, (size_t)nsv, 1, &slot));
  if (h->strength) {
    for (int64_t k = 0; k < nsv; ++k)
      TRY(upload_gather(h, h->d_statev + (size_t)(k * ne), s->elem_statev, t.elem_int2ext, (size_t)nsv, (size_t)k,
                        &slot));
    // reference bin rb -> device bin rb ^ 1, component i*3+j -> row i*3+j
    for (int rb = 0; rb < 2; ++rb)
      for (int k = 0; k < 9; ++k) {
        double* dst = h->d_stress[rb ^ 1] + (size_t)(k * ne);
        if (s->elem_stress)
          TRY(upload_gather(h, dst, s->elem_stress + (size_t)(rb * ne * 9), t.elem_int2ext, 9, (size_t)k, &slot));
        else
          CUDA_TRY(cudaMemsetAsync(dst, 0, sizeof(double) * (size_t)ne, h->stream));
      }
  }
  std::vector<int32_t> mat((size_t)ne);
  for (int64_t e = 0; e < ne; ++e) mat[e] = (int32_t)s->elem_mat_id[t.elem_int2ext[e]];
  TRY(upload_raw(h, h->d_mat, mat.data(), sizeof(int32_t) * (size_t)ne));
  // the caller's elem_div is what the reference shows before any stage runs
  if (s->elem_div) TRY(upload_gather(h, h->d_div[1], s->elem_div, t.elem_int2ext, 1, 0, &slot));
  else CUDA_TRY(cudaMemsetAsync(h->d_div[1], 0, sizeof(double) * (size_t)ne, h->stream));
  return finish_set_state(h, time_value, graphics_time, dt);
}

extern "C" int fierro_sgh_set_state(fierro_sgh* h, const fierro_sgh_state* s) {
  clear_error();
  NvtxRange nvtx_("fierro_sgh_set_state");
  if (!h) return set_error(FIERRO_EINVAL, "handle is NULL");
  return set_state_impl(h, s, 0.0, h->lp.graphics_dt_ival, h->dt_start);
}

// One store per page, in parallel, so that the pages of an output array exist
// before the GPU writes it (the array is overwritten completely afterwards).
static void populate(double* p, size_t bytes) {
  if (!p || bytes == 0) return;
  static const size_t page = (size_t)std::max(4096L, sysconf(_SC_PAGESIZE));
  char* c = reinterpret_cast<char*>(p);
  const int64_t n = (int64_t)((bytes + page - 1) / page);
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < n; ++k) *(volatile char*)(c + (size_t)k * page) = 0;
}

extern "C" int fierro_sgh_get_state(fierro_sgh* h, fierro_sgh_state* s) {
  clear_error();
  NvtxRange nvtx_("fierro_sgh_get_state");
  if (!h || !s) return set_error(FIERRO_EINVAL, "handle or state is NULL");
  if (!h->has_state) return set_error(FIERRO_EINVAL, "get_state before set_state");
  if (h->strength && s->elem_statev && s->num_state_vars != h->nsv)
    return set_error(FIERRO_EINVAL, "get_state: num_state_vars %lld, the handle holds %lld",
                     (long long)s->num_state_vars, (long long)h->nsv);
  long long cyc = 0;
  TRY(cycles_done(h, &cyc));
  const int c = bin_now(h, cyc);  // cycle-start bin of the current (or next) cycle
  // at a cycle boundary reference bin 1 is bin c; mid-cycle it is bin c^1
  const int b1 = (h->stage == 0) ? c : (c ^ 1);
  const int b0 = b1 ^ 1;
  const int64_t nn = h->nn, ne = h->ne;
  const HostTopo& t = h->topo;
  const int bins[2] = {b0, b1};
  // the divergence the last executed stage used (reference elem_div)
  const long long stages_done = cyc * h->rk_num_stages + h->stage;
  const int qb = stages_done == 0 ? 1 : (int)((stages_done - 1) & 1);
  if (h->dims == 2 && !h->direct_host) return rz::get_state(h, s, bins, qb);
  if (h->direct_host) {
    // the kernels write the caller's arrays: make their pages resident first
    // (a GPU fault per untouched page costs far more than a host store per page)
    const size_t nb = sizeof(double);
    const size_t D = h->dims == 2 ? 2 : 3;
    populate(s->node_coords, nb * nn * 2 * D);
    populate(s->node_vel, nb * nn * 2 * D);
    populate(s->node_mass, nb * nn);
    populate(s->elem_sie, nb * ne * 2);
    double* e1[] = {s->elem_den, s->elem_pres, s->elem_sspd, s->elem_vol, s->elem_div, s->elem_mass};
    for (double* p : e1) populate(p, nb * ne);
    populate(s->corner_force, nb * ne * (D == 2 ? 8 : 24));
    if (h->strength) populate(s->elem_statev, nb * ne * (size_t)h->nsv);
    // a gas-only handle's stress is zero: the host writes it while the GPU
    // writes the rest
    const bool host_zero = s->elem_stress && !h->strength;
    if (!host_zero) populate(s->elem_stress, nb * ne * 18);
    fierro_sgh_state sg = *s;
    if (host_zero) sg.elem_stress = nullptr;
    TRY(xfer::download_state(h, &sg, bins, qb, false));
    if (host_zero) zero_parallel(s->elem_stress, (size_t)ne * 18);
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return FIERRO_OK;
  }
  for (int rb = 0; rb < 2; ++rb)
    for (int d = 0; d < 3; ++d) {
      if (s->node_coords)
        TRY(download_scatter(h, s->node_coords + (size_t)rb * nn * 3, h->d_x[bins[rb]][d], t.node_int2ext, 3, d));
      if (s->node_vel)
        TRY(download_scatter(h, s->node_vel + (size_t)rb * nn * 3, h->d_v[bins[rb]][d], t.node_int2ext, 3, d));
    }
  if (s->elem_sie)
    for (int rb = 0; rb < 2; ++rb)
      TRY(download_scatter(h, s->elem_sie + (size_t)rb * ne, h->d_sie[bins[rb]], t.elem_int2ext, 1, 0));
  if (s->node_mass) TRY(download_scatter(h, s->node_mass, h->d_node_mass, t.node_int2ext, 1, 0));
  if (s->elem_den) TRY(download_scatter(h, s->elem_den, h->d_den, t.elem_int2ext, 1, 0));
  if (s->elem_pres) TRY(download_scatter(h, s->elem_pres, h->d_pres, t.elem_int2ext, 1, 0));
  if (s->elem_sspd) TRY(download_scatter(h, s->elem_sspd, h->d_sspd, t.elem_int2ext, 1, 0));
  if (s->elem_vol) TRY(download_scatter(h, s->elem_vol, h->d_vol, t.elem_int2ext, 1, 0));
  if (s->elem_div) TRY(download_scatter(h, s->elem_div, h->d_div[qb], t.elem_int2ext, 1, 0));
  if (s->elem_mass) TRY(download_scatter(h, s->elem_mass, h->d_elem_mass, t.elem_int2ext, 1, 0));
  if (s->elem_stress && h->strength) {
    for (int rb = 0; rb < 2; ++rb)
      for (int k = 0; k < 9; ++k)
        TRY(download_scatter(h, s->elem_stress + (size_t)(rb * ne * 9), h->d_stress[bins[rb]] + (size_t)(k * ne),
                             t.elem_int2ext, 9, (size_t)k));
  } else if (s->elem_stress) {
    std::memset(s->elem_stress, 0, sizeof(double) * (size_t)ne * 18);
  }
  if (s->elem_statev && h->strength)
    for (int64_t k = 0; k < h->nsv; ++k)
      TRY(download_scatter(h, s->elem_statev, h->d_statev + (size_t)(k * ne), t.elem_int2ext, (size_t)h->nsv,
                           (size_t)k));
  if (s->corner_force) {
    // device [lid*3+dim][e] -> reference [(E*8+lid)*3+dim]
    for (int r = 0; r < 24; ++r)
      TRY(download_scatter(h, s->corner_force, h->d_force + (size_t)r * ne, t.elem_int2ext, 24, (size_t)r));
  }
  return FIERRO_OK;
}

extern "C" int fierro_sgh_enqueue_cycles(fierro_sgh* h, int64_t cycles) {
  clear_error();
  NvtxRange nvtx_("fierro_sgh_enqueue_cycles");
  if (!h || !h->has_state) return set_error(FIERRO_EINVAL, "enqueue before set_state");
  if (h->stage != 0) return set_error(FIERRO_EINVAL, "a cycle is partly run; finish it with run_stages");
  for (int64_t i = 0; i < cycles; ++i) {
    const int c = (int)((h->base + h->enq_cycles) & 1);
    if (h->out) TRY(output_before_cycle(h, h->enq_cycles));
    CUDA_TRY(cudaGraphLaunch(h->graph[c], h->stream));
    if (h->out) TRY(output_after_cycle(h));
    h->enq_cycles++;
  }
  return FIERRO_OK;
}

extern "C" int fierro_sgh_synchronize(fierro_sgh* h) {
  clear_error();
  if (!h) return set_error(FIERRO_EINVAL, "handle is NULL");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  return check_status(h);
}

// Re-align the host's cycle parity with the device after a run that may have
// stopped early (stopped cycles do nothing, so the state stays put).
static int realign(fierro_sgh* h) {
  long long cyc = 0;
  TRY(cycles_done(h, &cyc));
  h->enq_cycles = cyc;
  return FIERRO_OK;
}

extern "C" int fierro_sgh_run(fierro_sgh* h, int64_t cycles, int64_t* cycles_run) {
  clear_error();
  NvtxRange nvtx_("fierro_sgh_run");
  if (!h || !h->has_state) return set_error(FIERRO_EINVAL, "run before set_state");
  long long before = 0;
  TRY(realign(h));
  before = h->enq_cycles;
  TRY(fierro_sgh_enqueue_cycles(h, cycles));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  TRY(realign(h));
  if (cycles_run) *cycles_run = h->enq_cycles - before;
  return check_status(h);
}

extern "C" int fierro_sgh_run_stages(fierro_sgh* h, int64_t stages) {
  clear_error();
  NvtxRange nvtx_("fierro_sgh_run_stages");
  if (!h || !h->has_state) return set_error(FIERRO_EINVAL, "run_stages before set_state");
  TRY(realign(h));
  for (int64_t i = 0; i < stages; ++i) {
    const int c = (int)((h->base + h->enq_cycles) & 1);
    if (h->stage == 0) enqueue_dt(h);
    enqueue_stage(h, c, h->stage);
    h->stage++;
    if (h->stage == h->rk_num_stages) {
      h->ks->end(h->d_ctrl, h->lp, h->stream);
      h->stage = 0;
      h->enq_cycles++;
    }
  }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (h->stage == 0) TRY(realign(h));
  return check_status(h);
}

extern "C" int fierro_sgh_run_timed(fierro_sgh* h, int64_t cycles, float* kernel_ms, float* total_ms,
                                    int64_t* cycles_run) {
  clear_error();
  NvtxRange nvtx_("fierro_sgh_run_timed");
  if (!h || !h->has_state) return set_error(FIERRO_EINVAL, "run before set_state");
  if (h->stage != 0) return set_error(FIERRO_EINVAL, "a cycle is partly run; finish it with run_stages");
  TRY(realign(h));
  const long long before = h->enq_cycles;
  const int L = (int)fierro_sgh_launches_per_cycle(h);
  const size_t nev = (size_t)cycles * (size_t)L + 1;
  std::vector<cudaEvent_t> ev(nev, nullptr);
  for (auto& e : ev) CUDA_TRY(cudaEventCreate(&e));
  size_t k = 0;
  CUDA_TRY(cudaEventRecord(ev[k++], h->stream));
  for (int64_t i = 0; i < cycles; ++i) {
    const int c = (int)((h->base + h->enq_cycles) & 1);
    enqueue_dt(h);
    CUDA_TRY(cudaEventRecord(ev[k++], h->stream));
    for (int s = 0; s < h->rk_num_stages; ++s) TRY(enqueue_stage_ev(h, c, s, ev.data(), &k));
    h->ks->end(h->d_ctrl, h->lp, h->stream);
    CUDA_TRY(cudaEventRecord(ev[k++], h->stream));
    h->enq_cycles++;
  }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaEventSynchronize(ev[k - 1]));
  if (kernel_ms)
    for (int i = 0; i < L; ++i) kernel_ms[i] = 0.0f;
  for (size_t j = 1; j < k; ++j) {
    float ms = 0.0f;
    CUDA_TRY(cudaEventElapsedTime(&ms, ev[j - 1], ev[j]));
    if (kernel_ms) kernel_ms[(j - 1) % (size_t)L] += ms;
  }
  if (total_ms) CUDA_TRY(cudaEventElapsedTime(total_ms, ev[0], ev[k - 1]));
  for (auto& e : ev) cudaEventDestroy(e);
  TRY(realign(h));
  if (cycles_run) *cycles_run = h->enq_cycles - before;
  return check_status(h);
}

extern "C" int fierro_sgh_time(fierro_sgh* h, double* time_value, double* dt, double* graphics_time,
                               int64_t* cycle) {
  clear_error();
  if (!h) return set_error(FIERRO_EINVAL, "handle is NULL");
  Ctrl c;
  CUDA_TRY(cudaMemcpyAsync(&c, h->d_ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (time_value) *time_value = c.time_value;
  if (dt) *dt = c.dt;
  if (graphics_time) *graphics_time = c.graphics_time;
  if (cycle) *cycle = c.cycle;
  return FIERRO_OK;
}

extern "C" int fierro_sgh_energy(fierro_sgh* h, double* ie, double* ke) {
  clear_error();
  NvtxRange nvtx_("fierro_sgh_energy");
  if (!h || !h->has_state) return set_error(FIERRO_EINVAL, "energy before set_state");
  long long cyc = 0;
  TRY(cycles_done(h, &cyc));
  const int c = bin_now(h, cyc);
  const int b1 = (h->stage == 0) ? c : (c ^ 1);
  if (h->dims == 2) return rz::energy(h, b1, ie, ke);
  EnergyArgs a{};
  a.ne = (int)h->ne;
  a.nn = (int)h->nn;
  a.mass = h->d_elem_mass;
  a.sie = h->d_sie[b1];
  a.node_mass = h->d_node_mass;
  a.u = h->d_v[b1][0];
  a.v = h->d_v[b1][1];
  a.w = h->d_v[b1][2];
  a.part = h->d_energy_part;
  a.out = h->d_energy_out;
  h->ks->energy(a, h->stream);
  double out[2];
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(out, h->d_energy_out, sizeof(out), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (ie) *ie = out[0];
  if (ke) *ke = out[1];
  return FIERRO_OK;
}

extern "C" int fierro_sgh_device_view(fierro_sgh* h, fierro_device_view* v) {
  clear_error();
  if (!h || !v) return set_error(FIERRO_EINVAL, "handle or view is NULL");
  if (!h->has_state) return set_error(FIERRO_EINVAL, "device_view before set_state");
  if (h->dims == 2) return set_error(FIERRO_ENOTSUP, "device_view: hex meshes only");
  if (h->stage != 0) return set_error(FIERRO_EINVAL, "device_view in the middle of a cycle");
  long long cyc = 0;
  TRY(cycles_done(h, &cyc));
  const int c = bin_now(h, cyc);
  std::memset(v, 0, sizeof(*v));
  v->num_nodes = h->nn;
  v->num_elems = h->ne;
  v->x = h->d_x[c][0];
  v->y = h->d_x[c][1];
  v->z = h->d_x[c][2];
  v->u = h->d_v[c][0];
  v->v = h->d_v[c][1];
  v->w = h->d_v[c][2];
  v->node_mass = h->d_node_mass;
  v->den = h->d_den;
  v->pres = h->d_pres;
  v->sspd = h->d_sspd;
  v->sie = h->d_sie[c];
  v->vol = h->d_vol;
  v->mass = h->d_elem_mass;
  const long long stages_done = cyc * h->rk_num_stages;
  v->div = h->d_div[stages_done == 0 ? 1 : (int)((stages_done - 1) & 1)];
  v->corner_force = h->d_force;
  v->node_int2ext = h->d_node_int2ext;
  v->elem_int2ext = h->d_elem_int2ext;
  v->node_ext2int = h->d_node_ext2int;
  v->elem_ext2int = h->d_elem_ext2int;
  v->stream = h->stream;
  return FIERRO_OK;
}

extern "C" int64_t fierro_sgh_launches_per_cycle(const fierro_sgh* h) {
  if (!h) return 0;
  return 2 + (h->dims == 2 ? 4 : 3) * (int64_t)h->rk_num_stages;
}

extern "C" int64_t fierro_sgh_device_bytes(const fierro_sgh* h) { return h ? (int64_t)h->dev_bytes : 0; }

extern "C" int fierro_sgh_solve(const fierro_mesh* mesh, const fierro_material* materials, int64_t num_materials,
                                const fierro_boundary* boundaries, int64_t num_bcs, fierro_sgh_state* state,
                                double* time_value, double time_final, double dt_max, double dt_min, double dt_cfl,
                                double* graphics_time, int64_t graphics_cyc_ival, double graphics_dt_ival,
                                int64_t cycle_stop, int64_t rk_num_stages, double dt, double fuzz, double tiny,
                                double small, int fp_mode, int64_t* cycles_run) {
  clear_error();
  NvtxRange nvtx_("fierro_sgh_solve");
  if (!time_value || !graphics_time || !state) return set_error(FIERRO_EINVAL, "solve: NULL argument");
  fierro_sgh_params p{time_final, dt_max, dt_min, dt_cfl, dt, graphics_dt_ival, graphics_cyc_ival,
                      cycle_stop, rk_num_stages, fuzz, tiny, small};
  fierro_sgh* h = nullptr;
  int rc = fierro_sgh_create(mesh, materials, num_materials, boundaries, num_bcs, &p, fp_mode, nullptr, &h);
  if (rc) return rc;
  rc = set_state_impl(h, state, *time_value, *graphics_time, dt);
  int64_t ran = 0;
  if (!rc) rc = fierro_sgh_run(h, cycle_stop, &ran);
  if (!rc) rc = fierro_sgh_get_state(h, state);
  if (!rc) rc = fierro_sgh_time(h, time_value, nullptr, graphics_time, nullptr);
  if (cycles_run) *cycles_run = ran;
  std::string msg = fierro_last_error();
  fierro_sgh_destroy(h);
  if (rc) set_error(rc, "%s", msg.c_str());
  return rc;
}

// ---------------------------------------------------------------------------
// Checkpoint / restart: everything the cycle loop carries from one cycle to the
// next, in the device numbering and bin roles, so a restarted loop continues
// bit for bit.  The reference has no restart; the nearest it has is calling
// sgh_solve again from the state the last call left, which restarts dt from
// dt_start (fierro_sgh_set_state does the same).
namespace {

// State variables per element a checkpoint may carry (the strength model reads
// kUserStrengthStateVars of them); larger counts in a header are refused as corrupt.
constexpr int64_t kMaxCheckpointStateVars = 4096;

struct CkptHeader {
  char magic[8];
  uint32_t version, dims;
  int64_t nn, ne, nsv, nmat, rk_num_stages, fp_mode, strength, topo_hash;
  int64_t base, ncfl;
};

struct Block {
  void* ptr;
  size_t bytes;
};

uint64_t fnv1a(uint64_t h, const void* p, size_t n) {
  const unsigned char* c = static_cast<const unsigned char*>(p);
  for (size_t i = 0; i < n; ++i) h = (h ^ c[i]) * 1099511628211ULL;
  return h;
}

// The device topology's fingerprint: connectivity, corner and neighbour lists
// and boundary masks in the device numbering.
uint64_t topo_hash(fierro_sgh* h) {
  const HostTopo& t = h->topo;
  uint64_t x = 1469598103934665603ULL;
  if (!t.nie.empty()) {
    x = fnv1a(x, t.nie.data(), t.nie.size() * sizeof(int32_t));
    x = fnv1a(x, t.cin.data(), t.cin.size() * sizeof(int32_t));
    x = fnv1a(x, t.eie.data(), t.eie.size() * sizeof(int32_t));
    x = fnv1a(x, t.bc_mask.data(), t.bc_mask.size());
    return x;
  }
  // topology built on the GPU (sgh_topo.cu): hash the device copies
  const size_t npe = h->dims == 2 ? 4 : 8;
  std::vector<int32_t> buf;
  auto add = [&](const int* d, size_t n) {
    buf.resize(std::max<size_t>(n, 1));
    if (n) cudaMemcpy(buf.data(), d, n * sizeof(int32_t), cudaMemcpyDeviceToHost);
    x = fnv1a(x, buf.data(), n * sizeof(int32_t));
  };
  add(h->d_nie, (size_t)h->ne * npe);
  add(h->d_cin, (size_t)h->ne * npe);
  add(h->d_eie, (size_t)h->nnz_eie);
  std::vector<unsigned char> bc((size_t)h->nn);
  cudaMemcpy(bc.data(), h->d_bc, bc.size(), cudaMemcpyDeviceToHost);
  return fnv1a(x, bc.data(), bc.size());
}

std::vector<Block> ckpt_blocks(fierro_sgh* h) {
  const size_t nn = (size_t)h->nn, ne = (size_t)h->ne, D = h->dims == 2 ? 2 : 3, d8 = sizeof(double);
  std::vector<Block> b;
  for (int bin = 0; bin < 2; ++bin)
    for (size_t d = 0; d < D; ++d) {
      b.push_back({h->d_x[bin][d], nn * d8});
      b.push_back({h->d_v[bin][d], nn * d8});
    }
  for (int bin = 0; bin < 2; ++bin) {
    b.push_back({h->d_sie[bin], ne * d8});
    b.push_back({h->d_div[bin], ne * d8});
  }
  for (double* p : {h->d_den, h->d_pres, h->d_sspd, h->d_vol, h->d_elem_mass, h->d_gamma, h->d_csmin})
    b.push_back({p, ne * d8});
  b.push_back({h->d_mat, ne * sizeof(int)});
  b.push_back({h->d_node_mass, nn * d8});
  b.push_back({h->d_force, ne * (h->dims == 2 ? 8 : 24) * d8});
  b.push_back({h->d_cfl, (size_t)h->ncfl * sizeof(long long)});
  b.push_back({h->d_ctrl, sizeof(Ctrl)});
  if (h->dims == 2) b.push_back({h->d_node_ext, nn * d8});
  else b.push_back({h->d_bmat, ne * 24 * d8});
  if (h->strength) {
    b.push_back({h->d_stress[0], ne * 9 * d8});
    b.push_back({h->d_stress[1], ne * 9 * d8});
    b.push_back({h->d_statev, ne * (size_t)h->nsv * d8});
  }
  return b;
}

CkptHeader ckpt_header(fierro_sgh* h) {
  CkptHeader hd{};
  std::memcpy(hd.magic, "FSGHCKPT", 8);
  hd.version = 1;
  hd.dims = (uint32_t)h->dims;
  hd.nn = h->nn;
  hd.ne = h->ne;
  hd.nsv = h->strength ? h->nsv : 0;
  hd.nmat = h->nmat;
  hd.rk_num_stages = h->rk_num_stages;
  hd.fp_mode = h->fp_mode;
  hd.strength = (h->strength ? 1 : 0) | (h->has_hyper ? 2 : 0);
  hd.topo_hash = (int64_t)topo_hash(h);
  hd.base = h->base;
  hd.ncfl = h->ncfl;
  return hd;
}

}  // namespace

extern "C" int fierro_sgh_checkpoint(fierro_sgh* h, const char* path) {
  clear_error();
  NvtxRange nvtx_("fierro_sgh_checkpoint");
  if (!h || !path) return set_error(FIERRO_EINVAL, "checkpoint: handle or path is NULL");
  if (!h->has_state) return set_error(FIERRO_EINVAL, "checkpoint before set_state");
  if (h->stage != 0) return set_error(FIERRO_EINVAL, "checkpoint in the middle of a cycle");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  TRY(check_status(h));
  TRY(realign(h));
  FILE* f = std::fopen(path, "wb");
  if (!f) return set_error(FIERRO_EINVAL, "checkpoint: cannot open %s for writing", path);
  const CkptHeader hd = ckpt_header(h);
  bool ok = std::fwrite(&hd, sizeof(hd), 1, f) == 1;
  std::vector<char> buf;
  for (const Block& b : ckpt_blocks(h)) {
    if (!ok) break;
    buf.resize(std::max<size_t>(b.bytes, 1));
    cudaError_t err = cudaMemcpy(buf.data(), b.ptr, b.bytes, cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) {
      std::fclose(f);
      return set_error(FIERRO_ECUDA, "checkpoint: %s", cudaGetErrorString(err));
    }
    ok = std::fwrite(buf.data(), 1, b.bytes, f) == b.bytes;
  }
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return set_error(FIERRO_EINVAL, "checkpoint: writing %s failed", path);
  return FIERRO_OK;
}

extern "C" int fierro_sgh_restart(fierro_sgh* h, const char* path) {
  clear_error();
  NvtxRange nvtx_("fierro_sgh_restart");
  if (!h || !path) return set_error(FIERRO_EINVAL, "restart: handle or path is NULL");
  FILE* f = std::fopen(path, "rb");
  if (!f) return set_error(FIERRO_EINVAL, "restart: cannot open %s", path);
  CkptHeader hd{};
  if (std::fread(&hd, sizeof(hd), 1, f) != 1 || std::memcmp(hd.magic, "FSGHCKPT", 8) != 0 || hd.version != 1) {
    std::fclose(f);
    return set_error(FIERRO_EINVAL, "restart: %s is not a checkpoint of this library", path);
  }
  // Every header field is checked against this handle, and the file's length
  // against the payload the header implies, before anything of the handle
  // changes: a refused file leaves the current state and graphs as they were.
  CkptHeader mine = ckpt_header(h);
  mine.base = hd.base;
  mine.nsv = hd.nsv;
  const bool nsv_ok = h->strength ? (hd.nsv >= kUserStrengthStateVars && hd.nsv <= kMaxCheckpointStateVars)
                                  : hd.nsv == 0;
  if (std::memcmp(&mine, &hd, sizeof(hd)) != 0 || !nsv_ok || (hd.base != 0 && hd.base != 1)) {
    std::fclose(f);
    return set_error(FIERRO_EINVAL, "restart: %s was written by a handle with another mesh, deck or parameters",
                     path);
  }
  size_t payload = 0;
  for (const Block& b : ckpt_blocks(h)) payload += b.bytes;
  if (h->strength) {
    const size_t ne = (size_t)h->ne;
    payload = payload - sizeof(double) * ne * (size_t)(h->d_statev ? h->nsv : 0) +
              sizeof(double) * ne * (size_t)hd.nsv;
  }
  if (std::fseek(f, 0, SEEK_END) != 0 || std::ftell(f) != (long)(sizeof(hd) + payload) ||
      std::fseek(f, (long)sizeof(hd), SEEK_SET) != 0) {
    std::fclose(f);
    return set_error(FIERRO_EINVAL, "restart: %s is truncated or longer than its header says", path);
  }
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (h->strength) {
    const int rc = size_statev(h, hd.nsv);
    if (rc) {
      std::fclose(f);
      return rc;
    }
  }
  h->has_state = false;
  if (h->adj) adj_release(h);
  output_reset(h);
  std::vector<char> buf;
  for (const Block& b : ckpt_blocks(h)) {
    buf.resize(std::max<size_t>(b.bytes, 1));
    if (std::fread(buf.data(), 1, b.bytes, f) != b.bytes) {
      std::fclose(f);
      return set_error(FIERRO_EINVAL, "restart: %s is truncated", path);
    }
    cudaError_t err = cudaMemcpy(b.ptr, buf.data(), b.bytes, cudaMemcpyHostToDevice);
    if (err != cudaSuccess) {
      std::fclose(f);
      return set_error(FIERRO_ECUDA, "restart: %s", cudaGetErrorString(err));
    }
  }
  std::fclose(f);
  if (h->d_node_rm) h->ks->reciprocal(h->d_node_mass, h->d_node_rm, (int)h->nn, h->stream);
  h->base = (int)hd.base;
  h->stage = 0;
  h->has_state = true;
  TRY(realign(h));
  return check_status(h);
}

extern "C" int fierro_sgh_status(fierro_sgh* h, uint32_t* flags) {
  clear_error();
  if (!h || !flags) return set_error(FIERRO_EINVAL, "handle or flags is NULL");
  Ctrl c;
  CUDA_TRY(cudaMemcpyAsync(&c, h->d_ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  *flags = c.status;
  return FIERRO_OK;
}
