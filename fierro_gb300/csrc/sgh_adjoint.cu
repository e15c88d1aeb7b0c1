// Discrete adjoint (reverse mode) of the SGH cycle, FP64, for sm_103a.
//
// Compiled with --fmad=false, like the exact cycle kernels: every forward value the
// reverse pass recomputes (corner-force viscosity terms, limiter, Mach switch, CFL
// minimum) comes out bit-identical to what the cycle kernels computed, so the
// reverse pass takes exactly the forward run's branches.  The adjoint's own sums
// have no parity target; they are deterministic (fixed orders, no atomics on
// floating-point values), and their reciprocals and reciprocal square roots are
// the ~2^-43 float-pair forms of sgh_common.cuh (fast_rcp, fast_rsqrt: one FP64
// operation each).
//
// Per RK stage the reverse pass is three launches, mirroring the forward ones in
// reverse order:
//   k_adj_elem   energy, divergence, volume and corner normals of the state the
//                stage produced -> per-corner node adjoints, power adjoint
//   k_adj_node   per-node gather of those corners; position / velocity update
//                and boundary conditions in reverse -> node force adjoint
//   k_adj_force  the corner force (MARS viscosity with the limiter, Mach switch
//                and compression branch frozen at the forward's choice) and the
//                equation of state of the stage's input state in reverse
// and per cycle k_adj_dt: the time-step choice (growth cap, CFL minimum through
// its minimising element and node pair, dt_min/dt_max, graphics and final-time
// clamps) and the time bookkeeping in reverse.
//
// Branch points are differentiated on their active side: |v - v_avg| and the
// divergence sign contribute zero at exactly zero (the symmetric derivative),
// the limiter's minimum goes to the first neighbour attaining it, the CFL
// minimum to the lowest-numbered element and first node pair attaining it.
#include <climits>
#include <cstdint>

#include "sgh_adjoint.h"

#define FIERRO_FMA 0

namespace fierro {
namespace adj_impl {

#include "sgh_common.cuh"
#include "sgh_hex_geometry.cuh"
#include "sgh_cfl.cuh"

constexpr int kAdjElemBlock = 128;
constexpr int kAdjForceBlock = 128;
constexpr int kAdjNodeBlock = 256;
constexpr long long kMaxKey = 0x7FFFFFFFFFFFFFFFLL;

enum { BR_GROW = 0, BR_CFL = 1, BR_DTMAX = 2, BR_DTMIN = 3, BR_GRAPH = 4, BR_FINAL = 5 };

// Block-wide sum, valid in thread 0; every thread of the block must call it.
__device__ __forceinline__ double block_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  __shared__ double ws[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) ws[wid] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  if (wid == 0) {
    v = lane < nw ? ws[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  }
  return v;
}

__device__ __forceinline__ void load_nodes(const int* nie, int e, int nid[8]) {
  const int4 n03 = __ldg(reinterpret_cast<const int4*>(nie) + 2 * e);
  const int4 n47 = __ldg(reinterpret_cast<const int4*>(nie) + 2 * e + 1);
  nid[0] = n03.x, nid[1] = n03.y, nid[2] = n03.z, nid[3] = n03.w;
  nid[4] = n47.x, nid[5] = n47.y, nid[6] = n47.z, nid[7] = n47.w;
}

// The dt choice of the cycle kernels' dt_update, re-derived from its recorded
// inputs; returns which candidate won.
__device__ __forceinline__ int dt_branch(double dt_prev, double time_value, double graphics_time, long long key,
                                         const LoopParams& lp, double* dt_out) {
  double dt = dt_prev * 1.1;
  const double raw = (key == kMaxKey) ? 1.7976931348623157e308 : okey_decode(key);
  double m = fmin(raw, lp.dt_max);
  m = fmax(m, lp.dt_min);
  int br = BR_GROW;
  if (m < dt) {
    dt = m;
    br = (raw < lp.dt_max && raw > lp.dt_min) ? BR_CFL : (m == lp.dt_max ? BR_DTMAX : BR_DTMIN);
  }
  const double g = (graphics_time - time_value) + lp.fuzz;
  if (g < dt) {
    dt = g;
    br = BR_GRAPH;
  }
  const double f = lp.time_final - time_value;
  if (f < dt) {
    dt = f;
    br = BR_FINAL;
  }
  *dt_out = dt;
  return br;
}

// Exact squared CFL length of one hex: min over the 28 node pairs, as order keys
// (equal to the screened evaluation of the cycle kernels, bit for bit); *pair
// receives the first pair attaining it.
__device__ __forceinline__ double min_pair_d2(const double* x, const double* y, const double* z, int* pair) {
  long long kmin = kMaxKey;
  int best = 0;
#pragma unroll
  for (int i = 0; i < 28; ++i) {
    const long long k = cfl::key_of(cfl::exact_d2(x, y, z, cfl::pair_a(i), cfl::pair_b(i)));
    if (k < kmin) {
      kmin = k;
      best = i;
    }
  }
  *pair = best;
  return cfl::key_decode(kmin);
}

// Reverse of the ideal-gas EOS (eos.cpp:12-46 as used by update_state):
// pres = (gamma - 1) sie den, sspd = max(sqrt(gamma (gamma - 1) sie), csmin).
__device__ __forceinline__ void eos_fold(double den, double sie, double gamma, double csmin, double presb,
                                         double sspdb, double& sieb, double& denb, double& gb) {
  sieb += presb * (gamma - 1.0) * den;
  denb += presb * (gamma - 1.0) * sie;
  gb += presb * sie * den;
  const double raw = sqrt(gamma * (gamma - 1.0) * sie);
  if (!(raw < csmin) && raw > 0.0) {
    const double t = sspdb * fast_rcp(2.0 * raw);
    sieb += t * gamma * (gamma - 1.0);
    gb += t * (2.0 * gamma - 1.0) * sie;
  }
}

// ---------------------------------------------------------------------------
// Forward-side helpers (run while the tape is recorded).

__global__ void k_adj_eos(int ne, const double* __restrict__ sie, const double* __restrict__ den,
                          const double* __restrict__ gamma, const double* __restrict__ csmin, double* __restrict__ pres,
                          double* __restrict__ sspd) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const double s = sie[e], g = gamma[e];
  pres[e] = (g - 1.0) * s * den[e];
  double c = sqrt(g * (g - 1.0) * s);
  if (c < csmin[e]) c = csmin[e];
  sspd[e] = c;
}

// Snapshot of the loop scalars and the CFL minimum before a cycle's dt kernel.
__global__ void __launch_bounds__(1024) k_adj_pre(AdjRecord* r, const long long* __restrict__ cfl_part, int nparts,
                                                  const Ctrl* ctrl) {
  long long k = kMaxKey;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
    const long long t = cfl_part[i];
    k = t < k ? t : k;
  }
  k = block_min_key(k);
  if (threadIdx.x == 0) {
    r->dt_prev = ctrl->dt;
    r->time_value = ctrl->time_value;
    r->graphics_time = ctrl->graphics_time;
    r->cfl_key = k;
    r->cycle = ctrl->cycle;
    r->estar = INT_MAX;
    r->dt = 0.0;
    r->active = 0;
  }
}

// After the dt kernel: the chosen dt, and (when the CFL minimum chose it) the
// lowest-numbered element whose CFL step equals the minimum.
__global__ void __launch_bounds__(kAdjElemBlock) k_adj_argmin(AdjRecord* r, const Ctrl* ctrl, const LoopParams lp,
                                                               const AdjMesh m, const Slot s) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e == 0) {
    r->dt = ctrl->dt;
    r->active = ctrl->active;
  }
  const long long key = r->cfl_key;
  double dtc;
  if (dt_branch(r->dt_prev, r->time_value, r->graphics_time, key, lp, &dtc) != BR_CFL || e >= m.ne) return;
  int nid[8];
  load_nodes(m.nie, e, nid);
  double x[8], y[8], z[8];
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    x[l] = s.x[nid[l]];
    y[l] = s.y[nid[l]];
    z[l] = s.z[nid[l]];
  }
  // screened exact minimum, as the element kernel evaluates it (same bits)
  __shared__ double s_xyz[24][kAdjElemBlock];
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    s_xyz[l][threadIdx.x] = x[l];
    s_xyz[8 + l][threadIdx.x] = y[l];
    s_xyz[16 + l][threadIdx.x] = z[l];
  }
  const double dist_min = sqrt(cfl::min_d2(x, y, z, &s_xyz[0][threadIdx.x], &s_xyz[8][threadIdx.x],
                                           &s_xyz[16][threadIdx.x], kAdjElemBlock));
  const double dt_l = lp.dt_cfl * dist_min / (s.sspd[e] + lp.fuzz);
  if (!isnan(dt_l) && okey(dt_l) == key) atomicMin(&r->estar, e);
}

// ---------------------------------------------------------------------------
// Seeds: adjoints of the final state's fields (den, pres, sspd fold through the
// EOS into sie and gamma, den into the volume).
__global__ void __launch_bounds__(256) k_adj_seed(const AdjMesh m, const AdjBufs b, const Slot f,
                                                  const double* __restrict__ eseed, const double* __restrict__ nseed,
                                                  unsigned mask, double* __restrict__ sb_next, const Node6 an) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int ne = m.ne, nn = m.nn;
  if (i == 0) {
    b.sc->dt_carry = 0.0;
    b.sc->time_bar = 0.0;
    b.sc->gtime_bar = 0.0;
    b.sc->status = 0u;
    b.sc->n_cfl = 0;
    b.sc->n_grow = 0;
    b.sc->n_other = 0;
  }
  if (i < ne) {
    const int e = i;
    const double den = f.den[e], vol = f.vol[e];
    double denb = (mask & 1u) ? eseed[e] : 0.0;
    const double presb = (mask & 2u) ? eseed[(size_t)ne + e] : 0.0;
    double sieb = (mask & 4u) ? eseed[2 * (size_t)ne + e] : 0.0;
    const double sspdb = (mask & 8u) ? eseed[3 * (size_t)ne + e] : 0.0;
    double volb = (mask & 16u) ? eseed[4 * (size_t)ne + e] : 0.0;
    double gb = 0.0;
    eos_fold(den, f.sie[e], m.gamma[e], m.csmin[e], presb, sspdb, sieb, denb, gb);
    volb -= denb * den * fast_rcp(vol);  // den = M / vol
    b.volbar[e] = volb;
    b.divbar[e] = 0.0;
    b.nbv[e] = 0.0;
    b.nbc[e] = -1;
#pragma unroll
    for (int r = 0; r < 24; ++r) {
      b.bbar[(size_t)r * ne + e] = 0.0;
      b.cv[(size_t)r * ne + e] = 0.0;
    }
    sb_next[e] = sieb;
    b.gbar[e] = gb;
  }
  if (i < nn) {
#pragma unroll
    for (int k = 0; k < 6; ++k) an.p[k][i] = ((mask >> (5 + k)) & 1u) ? nseed[(size_t)k * nn + i] : 0.0;
  }
}

// ---------------------------------------------------------------------------
// Element pass in reverse.  s1 is the state the stage produced; its derived
// adjoints (corner normals, volume, own divergence) were left by the force pass
// that consumed it, the neighbours' limiter terms are gathered here.
//   div = (Sx + Sy + Sz) / vol, S_c = sum_p vel(p,c) B(p,c)   (momentum.cpp:265-286)
//   vol = V(x), dV/dx_p = B_p                                   (geometry.cpp:238-310)
//   B = B(x)                                                    (geometry.cpp:40-234)
//   sie1 = sie0 - adt / M * sum_corners F . h                   (energy_sgh.cpp:16-52)
// KIND 2 is the uploaded state: its volume is an input, not the geometry's.
template <int KIND>
__global__ void __launch_bounds__(kAdjElemBlock) k_adj_elem(const AdjMesh m, const AdjBufs b, const Slot s1,
                                                             const double* __restrict__ force,
                                                             const AdjRecord* __restrict__ r, double alpha,
                                                             const double* __restrict__ sie_in,
                                                             double* __restrict__ sie_c, int assign,
                                                             double* __restrict__ part) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = e < m.ne;
  double adtb = 0.0;
  if (live) {
    const int ne = m.ne;
    int nid[8];
    load_nodes(m.nie, e, nid);
    double divb = b.divbar[e];
    const int k0 = m.eie_start[e], k1 = m.eie_start[e + 1];
    for (int k = k0; k < k1; ++k) {
      const int nb = __ldg(m.eie + k);
      if (b.nbc[nb] == e) divb += b.nbv[nb];
    }
    double volb = b.volbar[e];
    const double vol = s1.vol[e];
    const double iv = fast_rcp(vol);
    const double sb = divb * iv;
    double Bb[24], xb[8], yb[8], zb[8];
    double S = 0.0;
#pragma unroll
    for (int p = 0; p < 8; ++p) {
      const int n = nid[p];
      const double vel[3] = {s1.u[n], s1.v[n], s1.w[n]};
      double bp[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const size_t idx = (size_t)(p * 3 + c) * ne + e;
        bp[c] = s1.bmat[idx];
        S = fma(vel[c], bp[c], S);
        Bb[p * 3 + c] = fma(sb, vel[c], b.bbar[idx]);
        b.cv[idx] = fma(sb, bp[c], b.cv[idx]);
      }
      xb[p] = bp[0];
      yb[p] = bp[1];
      zb[p] = bp[2];
    }
    volb = fma(-divb * S, iv * iv, volb);
    const double vw = (KIND == 0) ? volb : 0.0;  // dV/dx_p = B_p
#pragma unroll
    for (int p = 0; p < 8; ++p) {
      xb[p] *= vw;
      yb[p] *= vw;
      zb[p] *= vw;
    }
    double x[8], y[8], z[8];
#pragma unroll
    for (int p = 0; p < 8; ++p) {
      x[p] = s1.x[nid[p]];
      y[p] = s1.y[nid[p]];
      z[p] = s1.z[nid[p]];
    }
    hex_bmatrix_adjoint(x, y, z, Bb, xb, yb, zb);
#pragma unroll
    for (int p = 0; p < 8; ++p) {
      b.cx[(size_t)(p * 3 + 0) * ne + e] = xb[p];
      b.cx[(size_t)(p * 3 + 1) * ne + e] = yb[p];
      b.cx[(size_t)(p * 3 + 2) * ne + e] = zb[p];
    }
    if (KIND == 0) {
      const double sieb = sie_in[e];
      if (assign) sie_c[e] = sieb;
      else sie_c[e] += sieb;
      const double M = m.elem_mass[e];
      double power = 0.0;
#pragma unroll
      for (int l = 0; l < 8; ++l) {
        const int n = nid[l];
        power = fma(force[(size_t)(l * 3 + 0) * ne + e], s1.hx[n],
                    fma(force[(size_t)(l * 3 + 1) * ne + e], s1.hy[n],
                        fma(force[(size_t)(l * 3 + 2) * ne + e], s1.hz[n], power)));
      }
      const double adt = alpha * r->dt;
      const double iM = sieb * fast_rcp(M);
      b.w[e] = -adt * iM;
      adtb = -power * iM;
    }
  }
  if (KIND == 0) {
    const double t = block_sum(adtb);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
  }
}

// ---------------------------------------------------------------------------
// Node pass in reverse (momentum.cpp:11-53, boundary.cpp:10-55, geometry.cpp:9-26):
//   f = sum_corners F, v1 = v0 + adt f / m, v1[d] = 0 on held components,
//   h = (v1 + v0) / 2, x1 = x0 + adt h.
// an_in: direct adjoints of x1, v1 from later cycles (last stage only);
// an_c: adjoints of the cycle-start x0, v0 (assigned by the last stage, then
// accumulated by the earlier ones).
__global__ void __launch_bounds__(kAdjNodeBlock) k_adj_node(const AdjMesh m, const AdjBufs b, const Slot s1,
                                                             const double* __restrict__ force,
                                                             const AdjRecord* __restrict__ r, double alpha,
                                                             const Node6 an_in, const Node6 an_c, int assign,
                                                             double* __restrict__ part) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = n < m.nn;
  double adtb = 0.0;
  if (live) {
    const size_t ne = (size_t)m.ne;
    double gx = 0.0, gy = 0.0, gz = 0.0, gu = 0.0, gv = 0.0, gw = 0.0;
    double f0 = 0.0, f1 = 0.0, f2 = 0.0, hb0 = 0.0, hb1 = 0.0, hb2 = 0.0;
    const int c0 = m.cin_start[n], c1 = m.cin_start[n + 1];
    for (int c = c0; c < c1; ++c) {
      const int cid = __ldg(m.cin + c);
      const int e = cid >> 3, l = cid & 7;
      const size_t i0 = (size_t)(l * 3) * ne + e, i1 = i0 + ne, i2 = i1 + ne;
      gx += b.cx[i0];
      gy += b.cx[i1];
      gz += b.cx[i2];
      gu += b.cv[i0];
      gv += b.cv[i1];
      gw += b.cv[i2];
      const double we = b.w[e];
      const double F0 = force[i0], F1 = force[i1], F2 = force[i2];
      f0 += F0;
      f1 += F1;
      f2 += F2;
      hb0 += we * F0;
      hb1 += we * F1;
      hb2 += we * F2;
    }
    if (an_in.p[0]) {
      gx += an_in.p[0][n];
      gy += an_in.p[1][n];
      gz += an_in.p[2][n];
      gu += an_in.p[3][n];
      gv += an_in.p[4][n];
      gw += an_in.p[5][n];
    }
    const double adt = alpha * r->dt;
    hb0 += adt * gx;
    hb1 += adt * gy;
    hb2 += adt * gz;
    adtb = gx * s1.hx[n] + gy * s1.hy[n] + gz * s1.hz[n];
    double vb0 = gu + 0.5 * hb0, vb1 = gv + 0.5 * hb1, vb2 = gw + 0.5 * hb2;
    const unsigned bc = m.bc[n];
    if (bc & 1u) vb0 = 0.0;
    if (bc & 2u) vb1 = 0.0;
    if (bc & 4u) vb2 = 0.0;
    const double u0b = 0.5 * hb0 + vb0, v0b = 0.5 * hb1 + vb1, w0b = 0.5 * hb2 + vb2;
    const double rmass = fast_rcp(m.node_mass[n]);
    b.fbar[0][n] = vb0 * adt * rmass;
    b.fbar[1][n] = vb1 * adt * rmass;
    b.fbar[2][n] = vb2 * adt * rmass;
    adtb += (vb0 * f0 + vb1 * f1 + vb2 * f2) * rmass;
    if (assign) {
      an_c.p[0][n] = gx;
      an_c.p[1][n] = gy;
      an_c.p[2][n] = gz;
      an_c.p[3][n] = u0b;
      an_c.p[4][n] = v0b;
      an_c.p[5][n] = w0b;
    } else {
      an_c.p[0][n] += gx;
      an_c.p[1][n] += gy;
      an_c.p[2][n] += gz;
      an_c.p[3][n] += u0b;
      an_c.p[4][n] += v0b;
      an_c.p[5][n] += w0b;
    }
  }
  const double t = block_sum(adtb);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// ---------------------------------------------------------------------------
// Corner force in reverse (force_sgh.cpp:35-394, 3D, strength none), with the
// EOS of its input state.  The viscosity intermediates come from the replay's
// force tape (written by the cycle kernel itself, so they are the forward's
// values); when b.mismatch is set the corner forces are rebuilt from them with
// the cycle kernel's operations and compared bit for bit with force_tape.
//   F_l = B_l p + phi mu_l (v* - v_l), mu_l = den (qa c + qb |v_l - v_avg|) |B_l|,
//   v* = sum mu_l v_l / sum mu_l (if sum mu_l > fuzz), phi = alpha phi0,
//   phi0 = 1 - max(0, min(1, r_face)), r_face = 0.9 (div_nb + small)/(div + small),
//   alpha = min(1, 20 vol^(1/3) |div| / (c + fuzz)).
__global__ void __launch_bounds__(kAdjForceBlock, 3) k_adj_force(const AdjMesh m, const AdjBufs b, const Slot s0,
                                                               const Slot s1, const double* __restrict__ force_tape,
                                                               const double* __restrict__ ft,
                                                               const int* __restrict__ fsel, double fuzz,
                                                               double small, double* __restrict__ sie_out,
                                                               int accumulate) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.ne) return;
  const int ne = m.ne;
  int nid[8];
  load_nodes(m.nie, e, nid);
  double vu[8], vv[8], vw[8];
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    vu[l] = s0.u[nid[l]];
    vv[l] = s0.v[nid[l]];
    vw[l] = s0.w[nid[l]];
  }
  const double den = s0.den[e], pres = s0.pres[e], sspd = s0.sspd[e], vol = s0.vol[e], div = s0.div[e];
  const double* q = m.qtab + 4 * m.mat[e];
  const bool compress = div < 0;
  const double qa = compress ? q[0] : q[1];
  const double qb = compress ? q[2] : q[3];
  double vs0 = 0.0, vs1 = 0.0, vs2 = 0.0;
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    vs0 = fma(0.125, vu[l], vs0);
    vs1 = fma(0.125, vv[l], vs1);
    vs2 = fma(0.125, vw[l], vs2);
  }
  const double* t = ft + e;
  double mu[8], mv[8];
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    mu[l] = t[(size_t)l * ne];
    mv[l] = t[(size_t)(8 + l) * ne];
  }
  const double vstar0 = t[(size_t)16 * ne], vstar1 = t[(size_t)17 * ne], vstar2 = t[(size_t)18 * ne];
  const double s3 = t[(size_t)19 * ne], phi0 = t[(size_t)20 * ne], araw = t[(size_t)21 * ne];
  const double c_length = t[(size_t)22 * ne], r_min = t[(size_t)23 * ne];
  const int sel = fsel[e];
  const bool use_vstar = s3 > fuzz;
  const double q1c = qa * sspd;
  const double D = div + small;
  const double alpha = fmin(1.0, araw);
  const double phi = alpha * phi0;
  if (b.mismatch) {
    unsigned bad = 0;
#pragma unroll
    for (int l = 0; l < 8; ++l) {
      const double pm = phi * mu[l];
      const double vst[3] = {vstar0, vstar1, vstar2}, vl[3] = {vu[l], vv[l], vw[l]};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const size_t idx = (size_t)(l * 3 + c) * ne + e;
        const double f = s0.bmat[idx] * pres + pm * (vst[c] - vl[c]);
        bad += (__double_as_longlong(f) != __double_as_longlong(force_tape[idx])) ? 1u : 0u;
      }
    }
    if (bad) atomicAdd(b.mismatch, (unsigned long long)bad);
  }

  // reverse (no parity target: multiply-adds fused, reciprocals shared).
  // Pass 1: force adjoint Fbar_l = fbar(node) + w h(node) -> pressure, phi, v*
  // adjoints and the mu_l adjoints of the viscous term; B's pressure term.
  const double we = b.w[e];
  double presb = 0.0, phib = 0.0, vsb0 = 0.0, vsb1 = 0.0, vsb2 = 0.0;
  double mub[8];
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    const int n = nid[l];
    const double F0 = fma(we, s1.hx[n], b.fbar[0][n]);
    const double F1 = fma(we, s1.hy[n], b.fbar[1][n]);
    const double F2 = fma(we, s1.hz[n], b.fbar[2][n]);
    const size_t i0 = (size_t)(l * 3) * ne + e, i1 = i0 + ne, i2 = i1 + ne;
    presb = fma(F0, s0.bmat[i0], fma(F1, s0.bmat[i1], fma(F2, s0.bmat[i2], presb)));
    b.bbar[i0] = F0 * pres;
    b.bbar[i1] = F1 * pres;
    b.bbar[i2] = F2 * pres;
    const double pm = phi * mu[l];
    const double g = fma(F0, vstar0 - vu[l], fma(F1, vstar1 - vv[l], F2 * (vstar2 - vw[l])));
    phib = fma(mu[l], g, phib);
    mub[l] = phi * g;
    vsb0 = fma(pm, F0, vsb0);
    vsb1 = fma(pm, F1, vsb1);
    vsb2 = fma(pm, F2, vsb2);
  }
  const double alphab = phib * phi0, phi0b = phib * alpha;
  double divb = 0.0, sspdb = 0.0, volb = 0.0, denb = 0.0;
  if (araw < 1.0) {
    const double inv = fast_rcp(sspd + fuzz);
    const double sg = div > 0.0 ? 1.0 : (div < 0.0 ? -1.0 : 0.0);
    const double a20 = 20.0 * alphab * inv;
    divb = a20 * c_length * sg;
    sspdb = -alphab * alpha * inv;
    volb = a20 * fabs(div) * c_length * fast_rcp(3.0 * vol);
  }
  int nbc = -1;
  double nbv = 0.0;
  if (sel >= 0) {
    const double rbD = -phi0b * fast_rcp(D);  // phi0 = 1 - r_face
    nbv = 0.9 * rbD;
    nbc = sel;
    divb = fma(-rbD, r_min, divb);
  }
  double sb0 = 0.0, sb1 = 0.0, sb2 = 0.0, s3b = 0.0;
  if (use_vstar) {
    const double is3 = fast_rcp(s3);
    sb0 = vsb0 * is3;
    sb1 = vsb1 * is3;
    sb2 = vsb2 * is3;
    s3b = -fma(vsb0, vstar0, fma(vsb1, vstar1, vsb2 * vstar2)) * is3;
  }
  // Pass 2: per corner, the velocity adjoint (viscous term, v*, |v_l - v_avg|)
  // and the |B_l| term of mu_l.
  double vss0 = 0.0, vss1 = 0.0, vss2 = 0.0, q1cb = 0.0;
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    const int n = nid[l];
    const double F0 = fma(we, s1.hx[n], b.fbar[0][n]);
    const double F1 = fma(we, s1.hy[n], b.fbar[1][n]);
    const double F2 = fma(we, s1.hz[n], b.fbar[2][n]);
    const double pm = phi * mu[l];
    double vb0 = fma(mu[l], sb0, -pm * F0);
    double vb1 = fma(mu[l], sb1, -pm * F1);
    double vb2 = fma(mu[l], sb2, -pm * F2);
    const double mubl = fma(sb0, vu[l], fma(sb1, vv[l], fma(sb2, vw[l], mub[l] + s3b)));
    const size_t i0 = (size_t)(l * 3) * ne + e, i1 = i0 + ne, i2 = i1 + ne;
    const double b0 = s0.bmat[i0], b1 = s0.bmat[i1], b2 = s0.bmat[i2];
    const double qB = fma(b0, b0, fma(b1, b1, b2 * b2));
    const double rB = fast_rsqrt(qB);
    const double nB = qB * rB;
    const double qm = fma(qb, mv[l], q1c);
    const double mucb = mubl * nB;
    const double t = mubl * den * qm * rB;  // d mu / d B_l = muc B_l / |B_l|
    b.bbar[i0] = fma(t, b0, b.bbar[i0]);
    b.bbar[i1] = fma(t, b1, b.bbar[i1]);
    b.bbar[i2] = fma(t, b2, b.bbar[i2]);
    denb = fma(mucb, qm, denb);
    q1cb = fma(mucb, den, q1cb);
    if (mv[l] > 0.0) {
      const double d0 = vu[l] - vs0, d1 = vv[l] - vs1, d2 = vw[l] - vs2;
      const double sm = mucb * den * qb * fast_rsqrt(fma(d0, d0, fma(d1, d1, d2 * d2)));
      vb0 = fma(sm, d0, vb0);
      vb1 = fma(sm, d1, vb1);
      vb2 = fma(sm, d2, vb2);
      vss0 = fma(-sm, d0, vss0);
      vss1 = fma(-sm, d1, vss1);
      vss2 = fma(-sm, d2, vss2);
    }
    b.cv[i0] = vb0;
    b.cv[i1] = vb1;
    b.cv[i2] = vb2;
  }
  sspdb = fma(q1cb, qa, sspdb);
  // Pass 3: the average velocity's adjoint reaches every corner equally.
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    const size_t i0 = (size_t)(l * 3) * ne + e;
    b.cv[i0] = fma(0.125, vss0, b.cv[i0]);
    b.cv[i0 + ne] = fma(0.125, vss1, b.cv[i0 + ne]);
    b.cv[i0 + 2 * (size_t)ne] = fma(0.125, vss2, b.cv[i0 + 2 * (size_t)ne]);
  }
  double sieb = 0.0, gb = 0.0;
  eos_fold(den, s0.sie[e], m.gamma[e], m.csmin[e], presb, sspdb, sieb, denb, gb);
  volb -= denb * den * fast_rcp(vol);  // den = M / vol
  b.volbar[e] = volb;
  b.divbar[e] = divb;
  b.nbc[e] = nbc;
  b.nbv[e] = nbv;
  if (accumulate) sie_out[e] += sieb;
  else sie_out[e] = sieb;
  b.gbar[e] += gb;
}

// ---------------------------------------------------------------------------
// dt and time bookkeeping of one cycle in reverse (time_integration.cpp:54-154,
// sgh_solve.cpp:590-632).  dt = rk_alpha-weighted sum of the stages' partial
// adjoints + the next cycle's growth-cap carry + the time adjoint.
__global__ void __launch_bounds__(1024) k_adj_dt(const AdjMesh m, const AdjBufs b, const AdjRecord* __restrict__ rp,
                                                 const LoopParams lp, const Slot s0, int stages, const AdjAlphas al,
                                                 const Node6 an_c, double* __restrict__ sie_c) {
  double acc = 0.0;
  for (int s = 0; s < stages; ++s) {
    double t = 0.0;
    for (int i = threadIdx.x; i < b.nbe; i += blockDim.x) t += b.part_e[(size_t)s * b.nbe + i];
    for (int i = threadIdx.x; i < b.nbn; i += blockDim.x) t += b.part_n[(size_t)s * b.nbn + i];
    acc += al.a[s] * t;
  }
  acc = block_sum(acc);
  if (threadIdx.x != 0) return;
  const AdjRecord r = *rp;
  AdjScalars* sc = b.sc;
  double dt_re;
  const int br = dt_branch(r.dt_prev, r.time_value, r.graphics_time, r.cfl_key, lp, &dt_re);
  if (__double_as_longlong(dt_re) != __double_as_longlong(r.dt)) sc->status |= FIERRO_ADJ_STATUS_DT_MISMATCH;
  const double t1 = r.time_value + r.dt;
  bool write = false;
  if ((r.cycle + 1) % lp.graphics_cyc_ival == 0 && r.cycle > 0) write = true;
  else if (t1 >= lp.time_final) write = true;
  else if (t1 >= r.graphics_time) write = true;
  double tb = sc->time_bar, gtb = sc->gtime_bar;
  if (write) {  // graphics_time = time_value + graphics_dt_ival
    tb += gtb;
    gtb = 0.0;
  }
  const double dtb = acc + sc->dt_carry + tb;  // time_value += dt
  double carry = 0.0;
  if (br == BR_CFL) sc->n_cfl++;
  else if (br == BR_GROW) sc->n_grow++;
  else sc->n_other++;
  if (br == BR_GROW) {
    carry = 1.1 * dtb;
  } else if (br == BR_GRAPH) {
    gtb += dtb;
    tb -= dtb;
  } else if (br == BR_FINAL) {
    tb -= dtb;
  } else if (br == BR_CFL) {
    const int e = r.estar;
    if (e >= 0 && e < m.ne) {
      int nid[8];
      load_nodes(m.nie, e, nid);
      double x[8], y[8], z[8];
      for (int l = 0; l < 8; ++l) {
        x[l] = s0.x[nid[l]];
        y[l] = s0.y[nid[l]];
        z[l] = s0.z[nid[l]];
      }
      int pair;
      const double d2 = min_pair_d2(x, y, z, &pair);
      const double dist = sqrt(d2);
      const double sspd = s0.sspd[e];
      const double cden = sspd + lp.fuzz;
      const double dt_l = lp.dt_cfl * dist / cden;
      const double distb = dtb * lp.dt_cfl / cden;
      const double sspdb = -dtb * dt_l / cden;
      if (dist > 0.0) {
        const int pa = cfl::pair_a(pair), pb = cfl::pair_b(pair);
        const double k2 = distb / dist;  // d dist / d dx = dx / dist
        const double dx = x[pb] - x[pa], dy = y[pb] - y[pa], dz = z[pb] - z[pa];
        an_c.p[0][nid[pb]] += k2 * dx;
        an_c.p[0][nid[pa]] -= k2 * dx;
        an_c.p[1][nid[pb]] += k2 * dy;
        an_c.p[1][nid[pa]] -= k2 * dy;
        an_c.p[2][nid[pb]] += k2 * dz;
        an_c.p[2][nid[pa]] -= k2 * dz;
      }
      double sieb = 0.0, denb = 0.0, gb = 0.0;
      eos_fold(s0.den[e], s0.sie[e], m.gamma[e], m.csmin[e], 0.0, sspdb, sieb, denb, gb);
      sie_c[e] += sieb;
      b.gbar[e] += gb;
    } else {
      sc->status |= FIERRO_ADJ_STATUS_DT_MISMATCH;
    }
  }
  sc->dt_carry = carry;
  sc->time_bar = tb;
  sc->gtime_bar = gtb;
}

// Velocity adjoint of the uploaded state: direct term plus the corner terms of
// its force and divergence.
__global__ void __launch_bounds__(256) k_adj_vel0(const AdjMesh m, const AdjBufs b, const Node6 an) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= m.nn) return;
  const size_t ne = (size_t)m.ne;
  double gu = an.p[3][n], gv = an.p[4][n], gw = an.p[5][n];
  for (int c = m.cin_start[n]; c < m.cin_start[n + 1]; ++c) {
    const int cid = m.cin[c];
    const size_t i0 = (size_t)((cid & 7) * 3) * ne + (cid >> 3);
    gu += b.cv[i0];
    gv += b.cv[i0 + ne];
    gw += b.cv[i0 + 2 * ne];
  }
  b.fbar[0][n] = gu;
  b.fbar[1][n] = gv;
  b.fbar[2][n] = gw;
}

// ---------------------------------------------------------------------------
// Branch record and frozen-branch forward.

// The first node pair attaining the CFL minimum of the recorded element.
__global__ void k_adj_pair(AdjRecord* r, const AdjMesh m, const Slot s) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int e = r->estar;
  r->pair = -1;
  if (e < 0 || e >= m.ne) return;
  int nid[8];
  load_nodes(m.nie, e, nid);
  double x[8], y[8], z[8];
  for (int l = 0; l < 8; ++l) {
    x[l] = s.x[nid[l]];
    y[l] = s.y[nid[l]];
    z[l] = s.z[nid[l]];
  }
  int pair;
  min_pair_d2(x, y, z, &pair);
  r->pair = pair;
}

// The time step of the frozen-branch forward (time_integration.cpp:54-154 with the
// recorded cycle's decisions): the growth cap of this run's previous dt, the CFL
// step of the recorded element and node pair in this run's state, the dt_max /
// dt_min bounds, or the graphics / final-time clamps of this run's time.  On the
// recorded trajectory itself it equals the cycle kernels' dt bit for bit.
__global__ void k_adj_dt_frozen(const AdjRecord* __restrict__ rp, Ctrl* c, const LoopParams lp, const AdjMesh m,
                                const Slot s) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (c->stopped) {
    c->active = 0;
    return;
  }
  const AdjRecord r = *rp;
  double dt_rec;
  const int br = dt_branch(r.dt_prev, r.time_value, r.graphics_time, r.cfl_key, lp, &dt_rec);
  double dt = dt_rec;
  if (br == BR_GROW) {
    dt = c->dt * 1.1;
  } else if (br == BR_CFL) {
    const int e = r.estar;
    if (e >= 0 && e < m.ne && r.pair >= 0 && r.pair < 28) {
      int nid[8];
      load_nodes(m.nie, e, nid);
      double x[8], y[8], z[8];
      for (int l = 0; l < 8; ++l) {
        x[l] = s.x[nid[l]];
        y[l] = s.y[nid[l]];
        z[l] = s.z[nid[l]];
      }
      const double d2 = cfl::exact_d2(x, y, z, cfl::pair_a(r.pair), cfl::pair_b(r.pair));
      dt = lp.dt_cfl * sqrt(d2) / (s.sspd[e] + lp.fuzz);
    }
  } else if (br == BR_DTMAX) {
    dt = lp.dt_max;
  } else if (br == BR_DTMIN) {
    dt = lp.dt_min;
  } else if (br == BR_GRAPH) {
    dt = (c->graphics_time - c->time_value) + lp.fuzz;
  } else if (br == BR_FINAL) {
    dt = lp.time_final - c->time_value;
  }
  c->dt = dt;
  c->active = 1;
}

// ---------------------------------------------------------------------------
static unsigned blocks_for(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

static void launch_eos(int ne, const double* sie, const double* den, const double* gamma, const double* csmin,
                       double* pres, double* sspd, cudaStream_t st) {
  k_adj_eos<<<blocks_for(ne, 256), 256, 0, st>>>(ne, sie, den, gamma, csmin, pres, sspd);
}
static void launch_pre(AdjRecord* r, const long long* cfl_part, int nparts, const Ctrl* ctrl, cudaStream_t st) {
  k_adj_pre<<<1, 1024, 0, st>>>(r, cfl_part, nparts, ctrl);
}
static void launch_argmin(AdjRecord* r, const Ctrl* ctrl, const LoopParams& lp, const AdjMesh& m, const Slot& s,
                          cudaStream_t st) {
  k_adj_argmin<<<blocks_for(m.ne, kAdjElemBlock), kAdjElemBlock, 0, st>>>(r, ctrl, lp, m, s);
}
static void launch_seed(const AdjMesh& m, const AdjBufs& b, const Slot& fin, const double* eseed,
                        const double* nseed, unsigned mask, double* sb_next, const Node6& an, cudaStream_t st) {
  const int n = m.ne > m.nn ? m.ne : m.nn;
  k_adj_seed<<<blocks_for(n, 256), 256, 0, st>>>(m, b, fin, eseed, nseed, mask, sb_next, an);
}
static void launch_elem(const AdjMesh& m, const AdjBufs& b, const Slot& s1, const double* force,
                        const AdjRecord* r, double alpha, const double* sie_in, double* sie_c, int assign,
                        double* part, int kind, cudaStream_t st) {
  const unsigned g = blocks_for(m.ne, kAdjElemBlock);
  if (kind == 2) k_adj_elem<2><<<g, kAdjElemBlock, 0, st>>>(m, b, s1, force, r, alpha, sie_in, sie_c, assign, part);
  else k_adj_elem<0><<<g, kAdjElemBlock, 0, st>>>(m, b, s1, force, r, alpha, sie_in, sie_c, assign, part);
}
static void launch_node(const AdjMesh& m, const AdjBufs& b, const Slot& s1, const double* force,
                        const AdjRecord* r, double alpha, const Node6& an_in, const Node6& an_c, int assign,
                        double* part, cudaStream_t st) {
  k_adj_node<<<blocks_for(m.nn, kAdjNodeBlock), kAdjNodeBlock, 0, st>>>(m, b, s1, force, r, alpha, an_in, an_c,
                                                                         assign, part);
}
static void launch_force(const AdjMesh& m, const AdjBufs& b, const Slot& s0, const Slot& s1,
                         const double* force_tape, const double* ft, const int* fsel, double fuzz, double small,
                         double* sie_out, int accumulate, cudaStream_t st) {
  k_adj_force<<<blocks_for(m.ne, kAdjForceBlock), kAdjForceBlock, 0, st>>>(m, b, s0, s1, force_tape, ft, fsel, fuzz,
                                                                            small, sie_out, accumulate);
}
static void launch_dt(const AdjMesh& m, const AdjBufs& b, const AdjRecord* r, const LoopParams& lp,
                      const Slot& s0, int stages, const AdjAlphas& al, const Node6& an_c, double* sie_c,
                      cudaStream_t st) {
  k_adj_dt<<<1, 1024, 0, st>>>(m, b, r, lp, s0, stages, al, an_c, sie_c);
}
static void launch_vel0(const AdjMesh& m, const AdjBufs& b, const Node6& an, cudaStream_t st) {
  k_adj_vel0<<<blocks_for(m.nn, 256), 256, 0, st>>>(m, b, an);
}
static void launch_pair(AdjRecord* r, const AdjMesh& m, const Slot& s, cudaStream_t st) {
  k_adj_pair<<<1, 32, 0, st>>>(r, m, s);
}
static void launch_dt_frozen(const AdjRecord* r, Ctrl* ctrl, const LoopParams& lp, const AdjMesh& m, const Slot& s,
                             cudaStream_t st) {
  k_adj_dt_frozen<<<1, 32, 0, st>>>(r, ctrl, lp, m, s);
}

}  // namespace adj_impl

const AdjLaunch& adjoint_kernels() {
  static const AdjLaunch k = {adj_impl::launch_eos,  adj_impl::launch_pre,   adj_impl::launch_argmin,
                              adj_impl::launch_seed, adj_impl::launch_elem,  adj_impl::launch_node,
                              adj_impl::launch_force, adj_impl::launch_dt,   adj_impl::launch_vel0,
                              adj_impl::launch_pair,  adj_impl::launch_dt_frozen};
  return k;
}

}  // namespace fierro
