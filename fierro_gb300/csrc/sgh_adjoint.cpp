// Discrete adjoint of the SGH cycle: checkpointing forward, tape replay and the
// reverse schedule behind fierro_adj_forward / fierro_adj_backward.
//
// Forward: the handle's own cycle graphs run the cycles (so the trajectory is the
// plain solver's, bit for bit); every k cycles the cycle-start state, the loop
// scalars and the CFL block minima are copied into a device-resident checkpoint.
// Backward, for each segment from the last: the checkpoint is restored into slot 0
// of the tape and the segment is replayed with the same cycle kernels, each stage
// writing its outputs into its own tape slot; then its cycles are reversed, three
// adjoint launches per stage and one per cycle (sgh_adjoint.cu).  The replay
// reproduces the forward bit for bit, so the reverse pass sees the forward's
// values and branches.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sgh_adjoint.h"
#include "sgh_handle.h"

using namespace fierro;
using namespace fierro::hd;

namespace fierro {

struct AdjState {
  int k = 0, S = 0, nseg_cap = 0;
  long long cycles = 0;  // cycles run by the last forward
  long long cyc0 = 0;    // handle cycle count when it started
  bool have_forward = false;
  bool verify = false;
  std::vector<void*> allocs;
  size_t bytes = 0, tape_bytes = 0, ckpt_bytes = 0;
  size_t slot_doubles = 0, ckpt_doubles = 0;
  double* tape = nullptr;    // (k*S + 1) slots
  double* forces = nullptr;  // k*S blocks of [24][ne]
  double* ftape = nullptr;   // k*S blocks of [kForceTapeRows][ne]
  int* fsel = nullptr;       // k*S blocks of [ne]
  double* ckpt = nullptr;    // nseg_cap checkpoints
  Ctrl* ckpt_ctrl = nullptr;
  long long* ckpt_cfl = nullptr;
  AdjRecord* rec = nullptr;  // k
  Ctrl* ctrl = nullptr;      // the replay's own loop scalars
  long long* cfl = nullptr;
  AdjMesh m{};
  AdjBufs b{};
  double* sb[2] = {};
  double* an[2][6] = {};
  double* eseed = nullptr;
  double* nseed = nullptr;
  unsigned long long* mismatch = nullptr;
  unsigned long long last_mismatch = 0;
  unsigned last_status = 0;
  int last_branches[3] = {0, 0, 0};  // CFL, growth cap, other
};

void adj_release(fierro_sgh* h) {
  if (!h || !h->adj) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (void* p : h->adj->allocs) cudaFree(p);
  delete h->adj;
  h->adj = nullptr;
}

// The branch decisions of one forward run (the base trajectory), cycle by cycle:
// per RK stage and element the corner force's branch bits and limiter neighbour,
// per cycle the time step's inputs, its CFL element and node pair.  A forward
// run in freeze mode takes every decision from here instead of deciding it.
struct AdjBranches {
  int mode = FIERRO_ADJ_BRANCHES_OFF;
  long long cycles = 0;      // cycles of the recorded run (0: nothing recorded yet)
  long long cap = 0;         // cycles the buffers hold
  int S = 0;
  int64_t ne = 0;
  unsigned char* flags = nullptr;  // [cap][S][ne]
  int* sel = nullptr;              // [cap][S][ne]
  AdjRecord* rec = nullptr;        // [cap]
  size_t bytes = 0;
};

void adj_branches_release(fierro_sgh* h) {
  if (!h || !h->adj_br) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  cudaFree(h->adj_br->flags);
  cudaFree(h->adj_br->sel);
  cudaFree(h->adj_br->rec);
  delete h->adj_br;
  h->adj_br = nullptr;
}

}  // namespace fierro

namespace {

template <typename T>
int aalloc(AdjState* a, T** p, size_t count) {
  void* q = nullptr;
  const size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
  cudaError_t err = cudaMalloc(&q, bytes);
  if (err != cudaSuccess)
    return set_error(FIERRO_ENOMEM, "adjoint: cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(err));
  a->allocs.push_back(q);
  a->bytes += bytes;
  *p = static_cast<T*>(q);
  return FIERRO_OK;
}

Slot slot_at(const fierro_sgh* h, const AdjState* a, long long j) {
  const size_t nn = (size_t)h->nn, ne = (size_t)h->ne;
  double* base = a->tape + (size_t)j * a->slot_doubles;
  Slot s;
  s.x = base;
  s.y = base + nn;
  s.z = base + 2 * nn;
  s.u = base + 3 * nn;
  s.v = base + 4 * nn;
  s.w = base + 5 * nn;
  s.hx = base + 6 * nn;
  s.hy = base + 7 * nn;
  s.hz = base + 8 * nn;
  double* eb = base + 9 * nn;
  s.sie = eb;
  s.vol = eb + ne;
  s.den = eb + 2 * ne;
  s.pres = eb + 3 * ne;
  s.sspd = eb + 4 * ne;
  s.div = eb + 5 * ne;
  s.bmat = eb + 6 * ne;
  return s;
}

double* force_at(const fierro_sgh* h, const AdjState* a, long long j) {
  return a->forces + (size_t)j * 24 * (size_t)h->ne;
}

Node6 node6(double* const p[6]) {
  Node6 n;
  for (int i = 0; i < 6; ++i) n.p[i] = p[i];
  return n;
}

// (Re)allocates the tape for `k` cycles and checkpoints for `nseg` segments.
int ensure(fierro_sgh* h, int k, int nseg) {
  const int S = h->rk_num_stages;
  AdjState* a = h->adj;
  if (a && a->k == k && a->S == S && a->nseg_cap >= nseg) return FIERRO_OK;
  adj_release(h);
  a = new (std::nothrow) AdjState();
  if (!a) return set_error(FIERRO_ENOMEM, "adjoint: host allocation failed");
  h->adj = a;
  a->k = k;
  a->S = S;
  a->nseg_cap = nseg;
  const size_t nn = (size_t)h->nn, ne = (size_t)h->ne;
  a->slot_doubles = 9 * nn + 30 * ne;
  a->ckpt_doubles = 6 * nn + 30 * ne;
  const size_t nslot = (size_t)k * S + 1;
  int rc = FIERRO_OK;
  auto fail = [&](int code) {
    std::string msg = fierro_last_error();
    adj_release(h);
    return set_error(code, "%s", msg.c_str());
  };
  if ((rc = aalloc(a, &a->tape, nslot * a->slot_doubles))) return fail(rc);
  if ((rc = aalloc(a, &a->forces, (size_t)k * S * 24 * ne))) return fail(rc);
  if ((rc = aalloc(a, &a->ftape, (size_t)k * S * kForceTapeRows * ne))) return fail(rc);
  if ((rc = aalloc(a, &a->fsel, (size_t)k * S * ne))) return fail(rc);
  a->tape_bytes = sizeof(double) * (nslot * a->slot_doubles + (size_t)k * S * (24 + kForceTapeRows) * ne) +
                  sizeof(int) * (size_t)k * S * ne;
  if ((rc = aalloc(a, &a->ckpt, (size_t)nseg * a->ckpt_doubles))) return fail(rc);
  if ((rc = aalloc(a, &a->ckpt_ctrl, (size_t)nseg))) return fail(rc);
  if ((rc = aalloc(a, &a->ckpt_cfl, (size_t)nseg * h->ncfl))) return fail(rc);
  a->ckpt_bytes = (size_t)nseg * (sizeof(double) * a->ckpt_doubles + sizeof(Ctrl) + sizeof(long long) * h->ncfl);
  if ((rc = aalloc(a, &a->rec, (size_t)k))) return fail(rc);
  if ((rc = aalloc(a, &a->ctrl, 1))) return fail(rc);
  if ((rc = aalloc(a, &a->cfl, (size_t)h->ncfl))) return fail(rc);
  AdjBufs& b = a->b;
  if ((rc = aalloc(a, &b.bbar, 24 * ne))) return fail(rc);
  if ((rc = aalloc(a, &b.cx, 24 * ne))) return fail(rc);
  if ((rc = aalloc(a, &b.cv, 24 * ne))) return fail(rc);
  if ((rc = aalloc(a, &b.volbar, ne))) return fail(rc);
  if ((rc = aalloc(a, &b.divbar, ne))) return fail(rc);
  if ((rc = aalloc(a, &b.nbv, ne))) return fail(rc);
  if ((rc = aalloc(a, &b.nbc, ne))) return fail(rc);
  if ((rc = aalloc(a, &b.w, ne))) return fail(rc);
  if ((rc = aalloc(a, &b.gbar, ne))) return fail(rc);
  if ((rc = aalloc(a, &b.sbt, ne))) return fail(rc);
  for (int d = 0; d < 3; ++d)
    if ((rc = aalloc(a, &b.fbar[d], nn))) return fail(rc);
  for (int i = 0; i < 2; ++i) {
    if ((rc = aalloc(a, &a->sb[i], ne))) return fail(rc);
    for (int d = 0; d < 6; ++d)
      if ((rc = aalloc(a, &a->an[i][d], nn))) return fail(rc);
  }
  b.nbe = (int)((ne + 127) / 128);
  b.nbn = (int)((nn + 255) / 256);
  if ((rc = aalloc(a, &b.part_e, (size_t)S * b.nbe))) return fail(rc);
  if ((rc = aalloc(a, &b.part_n, (size_t)S * b.nbn))) return fail(rc);
  if ((rc = aalloc(a, &b.sc, 1))) return fail(rc);
  if ((rc = aalloc(a, &a->mismatch, 1))) return fail(rc);
  if ((rc = aalloc(a, &a->eseed, 5 * ne))) return fail(rc);
  if ((rc = aalloc(a, &a->nseed, 6 * nn))) return fail(rc);
  AdjMesh& m = a->m;
  m.ne = (int)h->ne;
  m.nn = (int)h->nn;
  m.nie = h->d_nie;
  m.eie_start = h->d_eie_start;
  m.eie = h->d_eie;
  m.cin_start = h->d_cin_start;
  m.cin = h->d_cin;
  m.mat = h->d_mat;
  m.qtab = h->d_qtab;
  m.bc = h->d_bc;
  m.elem_mass = h->d_elem_mass;
  m.node_mass = h->d_node_mass;
  m.gamma = h->d_gamma;
  m.csmin = h->d_csmin;
  return FIERRO_OK;
}

// Copies the handle's cycle-start state (bin c) into checkpoint g.
int save_checkpoint(fierro_sgh* h, AdjState* a, int g, int c) {
  const size_t nn = (size_t)h->nn, ne = (size_t)h->ne;
  double* dst = a->ckpt + (size_t)g * a->ckpt_doubles;
  cudaStream_t st = h->stream;
  const size_t bn = sizeof(double) * nn, be = sizeof(double) * ne;
  for (int d = 0; d < 3; ++d) {
    CUDA_TRY(cudaMemcpyAsync(dst + d * nn, h->d_x[c][d], bn, cudaMemcpyDeviceToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(dst + (3 + d) * nn, h->d_v[c][d], bn, cudaMemcpyDeviceToDevice, st));
  }
  double* eb = dst + 6 * nn;
  const double* src[6] = {h->d_sie[c], h->d_vol, h->d_den, h->d_pres, h->d_sspd, h->d_div[div_parity(h, c, 0)]};
  for (int i = 0; i < 6; ++i) CUDA_TRY(cudaMemcpyAsync(eb + i * ne, src[i], be, cudaMemcpyDeviceToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(eb + 6 * ne, h->d_bmat, 24 * be, cudaMemcpyDeviceToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(a->ckpt_ctrl + g, h->d_ctrl, sizeof(Ctrl), cudaMemcpyDeviceToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(a->ckpt_cfl + (size_t)g * h->ncfl, h->d_cfl, sizeof(long long) * h->ncfl,
                           cudaMemcpyDeviceToDevice, st));
  return FIERRO_OK;
}

// Restores checkpoint g into tape slot 0 and replays n cycles, stage outputs
// into their own slots, recording each cycle's dt computation.
int replay_segment(fierro_sgh* h, AdjState* a, int g, int n) {
  const size_t nn = (size_t)h->nn, ne = (size_t)h->ne;
  cudaStream_t st = h->stream;
  const double* src = a->ckpt + (size_t)g * a->ckpt_doubles;
  CUDA_TRY(cudaMemcpyAsync(a->tape, src, sizeof(double) * 6 * nn, cudaMemcpyDeviceToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(a->tape + 9 * nn, src + 6 * nn, sizeof(double) * 30 * ne, cudaMemcpyDeviceToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(a->ctrl, a->ckpt_ctrl + g, sizeof(Ctrl), cudaMemcpyDeviceToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(a->cfl, a->ckpt_cfl + (size_t)g * h->ncfl, sizeof(long long) * h->ncfl,
                           cudaMemcpyDeviceToDevice, st));
  const AdjLaunch& K = adjoint_kernels();
  const int S = a->S;
  for (int i = 0; i < n; ++i) {
    const Slot c0 = slot_at(h, a, (long long)i * S);
    K.pre(a->rec + i, a->cfl, h->ncfl, a->ctrl, st);
    DtArgs d{};
    d.cfl_part = a->cfl;
    d.nparts = h->ncfl;
    d.ctrl = a->ctrl;
    d.lp = h->lp;
    h->ks->dt(d, st);
    K.argmin(a->rec + i, a->ctrl, h->lp, a->m, c0, st);
    for (int s = 0; s < S; ++s) {
      const long long j = (long long)i * S + s;
      const Slot sj = slot_at(h, a, j), sn = slot_at(h, a, j + 1);
      double* F = force_at(h, a, j);
      const double alpha = stage_alpha(h, s);
      ForceArgs fa{};
      fa.ne = (int)ne;
      fa.nie = h->d_nie;
      fa.eie_start = h->d_eie_start;
      fa.eie = h->d_eie;
      fa.mat = h->d_mat;
      fa.qtab = h->d_qtab;
      fa.bmat = sj.bmat;
      fa.u = sj.u;
      fa.v = sj.v;
      fa.w = sj.w;
      fa.den = sj.den;
      fa.pres = sj.pres;
      fa.sspd = sj.sspd;
      fa.vol = sj.vol;
      fa.div = sj.div;
      fa.force = F;
      fa.ctrl = a->ctrl;
      fa.fuzz = h->lp.fuzz;
      fa.small = h->lp.small;
      fa.tape = a->ftape + (size_t)j * kForceTapeRows * ne;
      fa.tape_sel = a->fsel + (size_t)j * ne;
      fa.block = h->blk_force;
      h->ks->force_tape(fa, st);
      NodeArgs na{};
      na.nn = (int)nn;
      na.ne = (int)ne;
      na.cin_start = h->d_cin_start;
      na.cin = h->d_cin;
      na.force = F;
      na.node_mass = h->d_node_mass;
      na.bc_mask = h->d_bc;
      na.u0 = c0.u;
      na.v0 = c0.v;
      na.w0 = c0.w;
      na.x0 = c0.x;
      na.y0 = c0.y;
      na.z0 = c0.z;
      na.u1 = sn.u;
      na.v1 = sn.v;
      na.w1 = sn.w;
      na.x1 = sn.x;
      na.y1 = sn.y;
      na.z1 = sn.z;
      na.hx = sn.hx;
      na.hy = sn.hy;
      na.hz = sn.hz;
      na.ctrl = a->ctrl;
      na.rk_alpha = alpha;
      na.block = h->blk_node;
      h->ks->node(na, st);
      ElemArgs ea{};
      ea.ne = (int)ne;
      ea.nie = h->d_nie;
      ea.x = sn.x;
      ea.y = sn.y;
      ea.z = sn.z;
      ea.u = sn.u;
      ea.v = sn.v;
      ea.w = sn.w;
      ea.hx = sn.hx;
      ea.hy = sn.hy;
      ea.hz = sn.hz;
      ea.force = F;
      ea.mass = h->d_elem_mass;
      ea.sie0 = c0.sie;
      ea.sie1 = sn.sie;
      ea.gamma = h->d_gamma;
      ea.csmin = h->d_csmin;
      ea.den = sn.den;
      ea.pres = sn.pres;
      ea.sspd = sn.sspd;
      ea.vol = sn.vol;
      ea.div = sn.div;
      ea.bmat = sn.bmat;
      ea.cfl_part = a->cfl;
      ea.ctrl = a->ctrl;
      ea.rk_alpha = alpha;
      ea.dt_cfl = h->lp.dt_cfl;
      ea.fuzz = h->lp.fuzz;
      ea.block = h->blk_elem;
      h->ks->elem(ea, s == S - 1 ? 1 : 0, st);
    }
    h->ks->end(a->ctrl, h->lp, st);
  }
  CUDA_TRY(cudaGetLastError());
  return FIERRO_OK;
}

AdjMesh mesh_of(const fierro_sgh* h) {
  AdjMesh m{};
  m.ne = (int)h->ne;
  m.nn = (int)h->nn;
  m.nie = h->d_nie;
  m.eie_start = h->d_eie_start;
  m.eie = h->d_eie;
  m.cin_start = h->d_cin_start;
  m.cin = h->d_cin;
  m.mat = h->d_mat;
  m.qtab = h->d_qtab;
  m.bc = h->d_bc;
  m.elem_mass = h->d_elem_mass;
  m.node_mass = h->d_node_mass;
  m.gamma = h->d_gamma;
  m.csmin = h->d_csmin;
  return m;
}

// The handle's state bin c as a tape slot (the fields the dt kernels read).
Slot bin_slot(const fierro_sgh* h, int c) {
  Slot s{};
  s.x = h->d_x[c][0];
  s.y = h->d_x[c][1];
  s.z = h->d_x[c][2];
  s.u = h->d_v[c][0];
  s.v = h->d_v[c][1];
  s.w = h->d_v[c][2];
  s.sie = h->d_sie[c];
  s.vol = h->d_vol;
  s.den = h->d_den;
  s.pres = h->d_pres;
  s.sspd = h->d_sspd;
  s.bmat = h->d_bmat;
  return s;
}

// Sizes the branch record for `cycles` cycles of this handle.
int branches_reserve(fierro_sgh* h, AdjBranches* br, long long cycles) {
  const int S = h->rk_num_stages;
  if (br->cap >= cycles && br->S == S && br->ne == h->ne) return FIERRO_OK;
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  cudaFree(br->flags);
  cudaFree(br->sel);
  cudaFree(br->rec);
  br->flags = nullptr;
  br->sel = nullptr;
  br->rec = nullptr;
  br->cap = br->cycles = 0;
  br->bytes = 0;
  const size_t n = (size_t)cycles * (size_t)S * (size_t)h->ne;
  cudaError_t e1 = cudaMalloc(&br->flags, std::max<size_t>(n, 1));
  cudaError_t e2 = e1 == cudaSuccess ? cudaMalloc(&br->sel, std::max<size_t>(n, 1) * sizeof(int)) : e1;
  cudaError_t e3 = e2 == cudaSuccess ? cudaMalloc(&br->rec, (size_t)cycles * sizeof(AdjRecord)) : e2;
  if (e3 != cudaSuccess) {
    cudaFree(br->flags);
    cudaFree(br->sel);
    br->flags = nullptr;
    br->sel = nullptr;
    br->rec = nullptr;
    return set_error(FIERRO_ENOMEM, "adjoint branch record for %lld cycles: %s", cycles, cudaGetErrorString(e3));
  }
  br->cap = cycles;
  br->S = S;
  br->ne = h->ne;
  br->bytes = n * (1 + sizeof(int)) + (size_t)cycles * sizeof(AdjRecord);
  return FIERRO_OK;
}

// One cycle of the handle's own schedule (the launches of its cycle graph) with
// the force passes recording (mode 1) or replaying (mode 2) cycle i of the
// branch record, and the time step recorded with its CFL element and node pair
// (mode 1) or taken along the recorded branch (mode 2).
void branch_cycle(fierro_sgh* h, AdjBranches* br, long long i, int mode) {
  const int c = (int)((h->base + h->enq_cycles) & 1);
  const int S = h->rk_num_stages;
  const size_t ne = (size_t)h->ne;
  const AdjLaunch& K = adjoint_kernels();
  const AdjMesh m = mesh_of(h);
  const Slot sc = bin_slot(h, c);
  AdjRecord* r = br->rec + i;
  if (mode == FIERRO_ADJ_BRANCHES_RECORD) {
    K.pre(r, h->d_cfl, h->ncfl, h->d_ctrl, h->stream);
    DtArgs d{};
    d.cfl_part = h->d_cfl;
    d.nparts = h->ncfl;
    d.ctrl = h->d_ctrl;
    d.lp = h->lp;
    h->ks->dt(d, h->stream);
    K.argmin(r, h->d_ctrl, h->lp, m, sc, h->stream);
    K.pair(r, m, sc, h->stream);
  } else {
    K.dt_frozen(r, h->d_ctrl, h->lp, m, sc, h->stream);
  }
  for (int s = 0; s < S; ++s) {
    ForceArgs fa = stage_force_args(h, c, s);
    fa.br_flags = br->flags + ((size_t)i * S + s) * ne;
    fa.br_sel = br->sel + ((size_t)i * S + s) * ne;
    h->ks->force_branch(fa, mode, h->stream);
    h->ks->node(node_args(h, c, stage_alpha(h, s)), h->stream);
    h->ks->elem(stage_elem_args(h, c, s), s == S - 1 ? 1 : 0, h->stream);
  }
  h->ks->end(h->d_ctrl, h->lp, h->stream);
}

int upload_seed(fierro_sgh* h, double* dst, const double* src, const std::vector<int64_t>& map, size_t stride,
                size_t off, int* slot) {
  return upload_gather(h, dst, src, map, stride, off, slot);
}

}  // namespace

extern "C" int fierro_adj_forward(fierro_sgh* h, const double* sie0, const double* gamma, int64_t cycles,
                                  int64_t ckpt_every, int64_t* cycles_run) {
  clear_error();
  NvtxRange nvtx_("fierro_adj_forward");
  if (cycles_run) *cycles_run = 0;
  if (!h || !h->has_state) return set_error(FIERRO_EINVAL, "adj_forward before set_state");
  if (h->stage != 0) return set_error(FIERRO_EINVAL, "adj_forward: a cycle is partly run");
  if (h->fp_mode != FIERRO_FP_EXACT)
    return set_error(FIERRO_ENOTSUP, "adj_forward: the adjoint differentiates the exact arithmetic mode only");
  if (h->strength)
    return set_error(FIERRO_ENOTSUP, "adj_forward: strength models are user code without a derivative");
  if (h->dims == 2) return set_error(FIERRO_ENOTSUP, "adj_forward: hex meshes only");
  if (cycles < 1 || ckpt_every < 1 || ckpt_every > (1 << 20))
    return set_error(FIERRO_EINVAL, "adj_forward: need cycles >= 1 and 1 <= ckpt_every <= 2^20");
  const int k = (int)std::min<int64_t>(ckpt_every, cycles);
  const long long nseg = (cycles + k - 1) / k;
  if (nseg > (1 << 24)) return set_error(FIERRO_EINVAL, "adj_forward: too many checkpoints");
  if (h->adj) h->adj->have_forward = false;
  AdjBranches* br = h->adj_br;
  const int bmode = br ? br->mode : FIERRO_ADJ_BRANCHES_OFF;
  if (bmode == FIERRO_ADJ_BRANCHES_FREEZE && (br->cycles != cycles || br->S != h->rk_num_stages || br->ne != h->ne))
    return set_error(FIERRO_EINVAL, "adj_forward: frozen branches were recorded for %lld cycles, %lld asked",
                     br->cycles, (long long)cycles);
  if (bmode == FIERRO_ADJ_BRANCHES_RECORD) TRY(branches_reserve(h, br, cycles));
  // the frozen-branch forward is a plain forward run: no checkpoints, and no
  // backward pass follows it
  AdjState* a = nullptr;
  if (bmode != FIERRO_ADJ_BRANCHES_FREEZE) {
    TRY(ensure(h, k, (int)nseg));
    a = h->adj;
  }
  long long cyc0 = 0;
  TRY(cycles_done(h, &cyc0));
  h->enq_cycles = cyc0;
  const int c = bin_now(h, cyc0);
  int slot = 0;
  const HostTopo& t = h->topo;
  if (sie0) TRY(upload_gather(h, h->d_sie[c], sie0, t.elem_int2ext, 1, 0, &slot));
  if (gamma) TRY(upload_gather(h, h->d_gamma, gamma, t.elem_int2ext, 1, 0, &slot));
  // pressure and sound speed of the parameters, then corner normals, divergence
  // and CFL minima of the resulting state
  adjoint_kernels().eos((int)h->ne, h->d_sie[c], h->d_den, h->d_gamma, h->d_csmin, h->d_pres, h->d_sspd, h->stream);
  h->ks->elem(elem_args(h, c, c, 1.0, div_parity(h, c, 0)), 2, h->stream);
  long long done = 0;
  for (long long g = 0; g < nseg; ++g) {
    if (a) TRY(save_checkpoint(h, a, (int)g, (int)((h->base + h->enq_cycles) & 1)));
    const long long n = std::min<long long>(k, cycles - g * k);
    for (long long i = 0; i < n; ++i, ++done) {
      if (bmode == FIERRO_ADJ_BRANCHES_OFF) CUDA_TRY(cudaGraphLaunch(h->graph[(h->base + h->enq_cycles) & 1], h->stream));
      else branch_cycle(h, br, done, bmode);
      h->enq_cycles++;
    }
  }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  long long cyc1 = 0;
  TRY(cycles_done(h, &cyc1));
  h->enq_cycles = cyc1;
  if (bmode == FIERRO_ADJ_BRANCHES_RECORD) br->cycles = cyc1 - cyc0 == cycles ? cycles : 0;
  if (cycles_run) *cycles_run = cyc1 - cyc0;
  if (a) {
    a->cyc0 = cyc0;
    a->cycles = cyc1 - cyc0;
    a->have_forward = a->cycles > 0;
  }
  return check_status(h);
}

extern "C" int fierro_adj_branches(fierro_sgh* h, int mode) {
  clear_error();
  if (!h) return set_error(FIERRO_EINVAL, "handle is NULL");
  if (mode == FIERRO_ADJ_BRANCHES_OFF) {
    adj_branches_release(h);
    return FIERRO_OK;
  }
  if (mode != FIERRO_ADJ_BRANCHES_RECORD && mode != FIERRO_ADJ_BRANCHES_FREEZE)
    return set_error(FIERRO_EINVAL, "adj_branches: mode %d is not OFF, RECORD or FREEZE", mode);
  if (h->fp_mode != FIERRO_FP_EXACT || h->strength || h->dims == 2)
    return set_error(FIERRO_ENOTSUP, "adj_branches: exact-mode gas-only hex handles only, as the adjoint");
  if (mode == FIERRO_ADJ_BRANCHES_FREEZE && (!h->adj_br || h->adj_br->cycles == 0))
    return set_error(FIERRO_EINVAL, "adj_branches: no recorded forward to freeze");
  if (!h->adj_br) {
    h->adj_br = new (std::nothrow) AdjBranches();
    if (!h->adj_br) return set_error(FIERRO_ENOMEM, "adj_branches: host allocation failed");
  }
  h->adj_br->mode = mode;
  return FIERRO_OK;
}

extern "C" int fierro_adj_backward(fierro_sgh* h, const fierro_adj_seed* seed, double* sie0_bar, double* gamma_bar,
                                   double* vel0_bar) {
  clear_error();
  NvtxRange nvtx_("fierro_adj_backward");
  if (!h || !h->adj || !h->adj->have_forward) return set_error(FIERRO_EINVAL, "adj_backward before adj_forward");
  AdjState* a = h->adj;
  long long cyc = 0;
  TRY(cycles_done(h, &cyc));
  if (cyc != a->cyc0 + a->cycles || h->stage != 0)
    return set_error(FIERRO_EINVAL, "adj_backward: the state changed since adj_forward");
  const HostTopo& t = h->topo;
  const size_t nn = (size_t)h->nn, ne = (size_t)h->ne;
  cudaStream_t st = h->stream;
  // seeds, device order
  unsigned mask = 0;
  int slot = 0;
  if (seed) {
    const double* es[5] = {seed->den, seed->pres, seed->sie, seed->sspd, seed->vol};
    for (int i = 0; i < 5; ++i)
      if (es[i]) {
        TRY(upload_seed(h, a->eseed + i * ne, es[i], t.elem_int2ext, 1, 0, &slot));
        mask |= 1u << i;
      }
    const double* ns[2] = {seed->coords, seed->vel};
    for (int i = 0; i < 2; ++i)
      if (ns[i]) {
        for (int d = 0; d < 3; ++d) TRY(upload_seed(h, a->nseed + (3 * i + d) * nn, ns[i], t.node_int2ext, 3, d, &slot));
        mask |= 7u << (5 + 3 * i);
      }
  }
  const AdjLaunch& K = adjoint_kernels();
  AdjBufs b = a->b;
  b.mismatch = a->verify ? a->mismatch : nullptr;
  if (a->verify) CUDA_TRY(cudaMemsetAsync(a->mismatch, 0, sizeof(unsigned long long), st));
  const int S = a->S, k = a->k;
  AdjAlphas al{};
  for (int s = 0; s < S; ++s) al.a[s] = stage_alpha(h, s);
  const long long nseg = (a->cycles + k - 1) / k;
  const Node6 none{{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr}};
  int p = 0;
  for (long long g = nseg - 1; g >= 0; --g) {
    const int n = (int)((g == nseg - 1) ? a->cycles - g * k : k);
    TRY(replay_segment(h, a, (int)g, n));
    if (g == nseg - 1)
      K.seed(a->m, b, slot_at(h, a, (long long)n * S), a->eseed, a->nseed, mask, a->sb[p], node6(a->an[p]), st);
    for (int i = n - 1; i >= 0; --i) {
      const Node6 an_n = node6(a->an[p]), an_c = node6(a->an[p ^ 1]);
      for (int s = S - 1; s >= 0; --s) {
        const long long j = (long long)i * S + s;
        const Slot sj = slot_at(h, a, j), sn = slot_at(h, a, j + 1);
        const double* F = force_at(h, a, j);
        const bool last = (s == S - 1);
        K.elem(a->m, b, sn, F, a->rec + i, al.a[s], last ? a->sb[p] : b.sbt, a->sb[p ^ 1], last ? 1 : 0,
               b.part_e + (size_t)s * b.nbe, 0, st);
        K.node(a->m, b, sn, F, a->rec + i, al.a[s], last ? an_n : none, an_c, last ? 1 : 0,
               b.part_n + (size_t)s * b.nbn, st);
        K.force(a->m, b, sj, sn, F, a->ftape + (size_t)j * kForceTapeRows * ne, a->fsel + (size_t)j * ne,
                h->lp.fuzz, h->lp.small, s > 0 ? b.sbt : a->sb[p ^ 1], s == 0 ? 1 : 0, st);
      }
      K.dt(a->m, b, a->rec + i, h->lp, slot_at(h, a, (long long)i * S), S, al, an_c, a->sb[p ^ 1], st);
      p ^= 1;
    }
    CUDA_TRY(cudaGetLastError());
  }
  // the uploaded state: its divergence used the uploaded volume
  K.elem(a->m, b, slot_at(h, a, 0), nullptr, nullptr, 0.0, nullptr, nullptr, 0, nullptr, 2, st);
  K.vel0(a->m, b, node6(a->an[p]), st);
  CUDA_TRY(cudaGetLastError());
  if (sie0_bar) TRY(download_scatter(h, sie0_bar, a->sb[p], t.elem_int2ext, 1, 0));
  if (gamma_bar) TRY(download_scatter(h, gamma_bar, b.gbar, t.elem_int2ext, 1, 0));
  if (vel0_bar)
    for (int d = 0; d < 3; ++d) TRY(download_scatter(h, vel0_bar, b.fbar[d], t.node_int2ext, 3, d));
  AdjScalars sc{};
  CUDA_TRY(cudaMemcpyAsync(&sc, b.sc, sizeof(sc), cudaMemcpyDeviceToHost, st));
  a->last_mismatch = 0;
  if (a->verify) CUDA_TRY(cudaMemcpyAsync(&a->last_mismatch, a->mismatch, sizeof(unsigned long long),
                                          cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  a->last_status = sc.status;
  a->last_branches[0] = sc.n_cfl;
  a->last_branches[1] = sc.n_grow;
  a->last_branches[2] = sc.n_other;
  if (sc.status & FIERRO_ADJ_STATUS_DT_MISMATCH)
    return set_error(FIERRO_ENUMERIC, "adj_backward: the replay's time steps differ from the forward's");
  if (a->last_mismatch)
    return set_error(FIERRO_ENUMERIC, "adj_backward: %llu recomputed corner forces differ from the replay's",
                     a->last_mismatch);
  return FIERRO_OK;
}

extern "C" int fierro_adj_verify(fierro_sgh* h, int enable) {
  clear_error();
  if (!h || !h->adj) return set_error(FIERRO_EINVAL, "adj_verify before adj_forward");
  h->adj->verify = enable != 0;
  return FIERRO_OK;
}

extern "C" int fierro_adj_stats(const fierro_sgh* h, int64_t* out, int64_t n) {
  if (!h || !out) return FIERRO_EINVAL;
  const AdjState* a = h->adj;
  const int64_t v[11] = {a ? a->cycles : 0,
                        a ? a->k : 0,
                        a ? (a->cycles + std::max(a->k, 1) - 1) / std::max(a->k, 1) : 0,
                        a ? (int64_t)a->tape_bytes : 0,
                        a ? (int64_t)a->ckpt_bytes : 0,
                        a ? (int64_t)a->bytes : 0,
                        a ? (int64_t)a->last_mismatch : 0,
                        a ? (int64_t)a->last_status : 0,
                        a ? a->last_branches[0] : 0,
                        a ? a->last_branches[1] : 0,
                        a ? a->last_branches[2] : 0};
  for (int64_t i = 0; i < n && i < 11; ++i) out[i] = v[i];
  return FIERRO_OK;
}

extern "C" int fierro_adj_release(fierro_sgh* h) {
  clear_error();
  if (!h) return set_error(FIERRO_EINVAL, "handle is NULL");
  adj_release(h);
  return FIERRO_OK;
}
