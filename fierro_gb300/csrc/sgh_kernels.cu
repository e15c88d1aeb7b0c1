// SGH cycle kernels for sm_103a (GB300), FP64.
//
// Compiled twice from this one source:
//   FIERRO_FMA=0 with --fmad=false -> fierro::exact_impl: every floating-point
//       operation is the reference's operation on the reference's operands in
//       the reference's order (Explicit-Lagrange-Kokkos/SGH_solver), with IEEE
//       division and square root, so results match its uncontracted evaluation;
//   FIERRO_FMA=1 with --fmad=true  -> fierro::fma_impl: the same schedule, the
//       compiler free to fuse multiply-adds, the per-node division by mass and
//       the Riemann velocity's three divisions done through one reciprocal
//       each, square and cube roots (within an ulp) and the remaining quotients
//       (the IEEE quotient's bits) by Newton iterations from single-precision
//       seeds, mostly on the FP32 and integer pipes (mode_sqrt, mode_cbrt,
//       mode_div, mode_rcp in sgh_common.cuh) -- except where the
//       reference's sums cancel (the hex volume, the element power, the Riemann
//       velocity), which stay separately rounded (FX_MUL / FX_ADD) so this mode
//       keeps within 1e-12 of the reference after one cycle and 1e-9 after a
//       full run.
//
// One cycle is 2 + 3*rk_num_stages launches:
//   k_dt                    CFL minimum over the last stage's per-block partials,
//                           dt growth/clamps (time_integration.cpp:54-154)
//   per RK stage s:
//     k_force   (elements)  MARS corner forces (force_sgh.cpp:12-399) from the
//                           corner normals the previous element pass stored
//     k_node    (nodes)     corner-force gather in the reference's summation order,
//                           velocity update, boundary conditions, position update
//                           (momentum.cpp:11-53, boundary.cpp:10-55, geometry.cpp:9-26)
//     k_elem    (elements)  energy (energy_sgh.cpp:6-55), volume (geometry.cpp:238-310),
//                           density/EOS (properties.cpp:9-114, eos.cpp:12-46), then
//                           the corner normals and divergence the NEXT stage starts
//                           from (momentum.cpp:221-292), and on the last stage the
//                           per-element CFL time step of the next cycle
//   k_end                   time advance, graphics-time bookkeeping, stop test
//                           (sgh_solve.cpp:590-632)
// rk_init's copies (time_integration.cpp:9-44) are replaced by swapping the roles
// of two state bins.  Nothing is accumulated with atomics: every output has one
// writer and every reduction has a fixed order.  A batch may instead run each
// RK stage as one cooperative launch of k_stage_fused (the three passes with
// grid barriers between them).
#include <algorithm>
#include <cstdint>

#include "sgh_device.h"

#ifndef FIERRO_FMA
#error "compile with -DFIERRO_FMA=0 or -DFIERRO_FMA=1"
#endif

#if FIERRO_FMA
#define FIERRO_IMPL fma_impl
#else
#define FIERRO_IMPL exact_impl
#endif

// Launch bounds of the force and element kernels.  FIERRO_FORCE_MIN_BLOCKS /
// FIERRO_ELEM_MIN_BLOCKS, when defined, ask the compiler for that many resident
// blocks per SM (a register budget of 65536 / (blocks x 128 threads)); undefined,
// the register count is the compiler's own choice.
#ifdef FIERRO_FORCE_MIN_BLOCKS
#define FIERRO_FORCE_BOUNDS __launch_bounds__(kForceBlock, FIERRO_FORCE_MIN_BLOCKS)
#else
#define FIERRO_FORCE_BOUNDS __launch_bounds__(kForceBlock)
#endif
#ifdef FIERRO_ELEM_MIN_BLOCKS
#define FIERRO_ELEM_BOUNDS __launch_bounds__(kElemBlock, FIERRO_ELEM_MIN_BLOCKS)
#else
#define FIERRO_ELEM_BOUNDS __launch_bounds__(kElemBlock)
#endif

// Corners whose force loads the node update issues together (FIERRO_NODE_GATHER
// overrides): eight in the FMA mode, four in the exact mode, where eight
// measured slower (256^3: FMA 1.66 -> 1.52 ms per launch with eight, exact
// 2.19 -> 2.26 ms).  The sums keep the corner order either way.
#ifndef FIERRO_NODE_GATHER
#define FIERRO_NODE_GATHER (FIERRO_FMA ? 8 : 4)
#endif

namespace fierro {
namespace FIERRO_IMPL {

constexpr int kNodeGather = FIERRO_NODE_GATHER;

// Loads of values an earlier phase of the same launch wrote (the batch's fused
// stage kernel, COH): from L2 (ld.global.cg), never from a line another phase
// left in this SM's L1.  Otherwise the read-only path (__ldg) or a plain load.
template <bool COH>
__device__ __forceinline__ double ld_ro(const double* p) {
  return COH ? __ldcg(p) : __ldg(p);
}
template <bool COH>
__device__ __forceinline__ double ld_pl(const double* p) {
  return COH ? __ldcg(p) : *p;
}

#include "sgh_common.cuh"
#include "sgh_hex_geometry.cuh"
#include "sgh_cfl.cuh"
#include "sgh_user_mat.cuh"

// Velocity gradient (momentum.cpp:59-144): L(i,j) = (sum_l v_i(l) B(l,j)) / vol,
// B the outward corner normals in rows [lid*3+dim][ne], summed over l in order.
__device__ __forceinline__ void velocity_gradient(const double (&u)[8], const double (&v)[8], const double (&w)[8],
                                                  const double* bmat, int ne, int e, double vol, double (&L)[9]) {
  const double inverse_vol = mode_rcp(vol);
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    double b = bmat[(size_t)j * ne + e];
    double su = u[0] * b, sv = v[0] * b, sw = w[0] * b;
#pragma unroll
    for (int l = 1; l < 8; ++l) {
      b = bmat[(size_t)(l * 3 + j) * ne + e];
      su = su + u[l] * b;
      sv = sv + v[l] * b;
      sw = sw + w[l] * b;
    }
    L[j] = su * inverse_vol;
    L[3 + j] = sv * inverse_vol;
    L[6 + j] = sw * inverse_vol;
  }
}

// ---------------------------------------------------------------------------
// Corner forces (force_sgh.cpp:35-394, 3D).  The reference's shock-direction
// and curl terms only feed unused values (use_shock_dir = 0 at :227, phi_curl
// unused at :331) and are not computed.  Without strength materials stress is
// zero, so tau = -p I and the force's stress term a_k tau(k,d) reduces exactly
// to B(d) p (two negations).  STRENGTH (a handle with a strength material)
// forms tau = stress(1) - p I and the force as the reference writes it, then
// runs the hypo model (:366-391) with the velocity gradient of this state.
// TAPE (the adjoint's replay, exact mode) also stores the viscosity
// intermediates; the stores do not change any value the kernel computes.
// BR = 1 records the element's branch decisions (compression sign, Riemann
// velocity, limiter case and neighbour, Mach clamp) without changing any value;
// BR = 2 takes them from the record instead of deciding them, so the force is a
// smooth function of the state along the recorded trajectory's branches.
template <bool BATCH, bool TAPE, bool STRENGTH, int BR>
__device__ __forceinline__ void force_elem(const ForceArgs& a, const int e) {
  if (BATCH && (a.inst[e] < 0 || !a.ctrl[a.inst[e]].active)) return;
  const int ne = a.ne;
  const int4 n03 = __ldg(reinterpret_cast<const int4*>(a.nie) + 2 * e);
  const int4 n47 = __ldg(reinterpret_cast<const int4*>(a.nie) + 2 * e + 1);
  const int nid[8] = {n03.x, n03.y, n03.z, n03.w, n47.x, n47.y, n47.z, n47.w};
  double vu[8], vv[8], vw[8];
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    vu[l] = __ldg(a.u + nid[l]);
    vv[l] = __ldg(a.v + nid[l]);
    vw[l] = __ldg(a.w + nid[l]);
  }
  const double den = a.den[e], pres = a.pres[e], sspd = a.sspd[e], vol = a.vol[e], div = a.div[e];
  const int mat = a.mat[e];
  const double* q = a.qtab + 4 * mat;
  const unsigned br = BR == 2 ? (unsigned)a.br_flags[e] : 0u;
  const bool compress = BR == 2 ? (br & FIERRO_BR_COMPRESS) != 0 : div < 0;
  const double qa = compress ? q[0] : q[1];  // q1 or q1ex
  const double qb = compress ? q[2] : q[3];  // q2 or q2ex

  // average velocity, the first Riemann-velocity estimate (:147-164); 0.125*v is
  // exact, so the fused form equals the reference's product-then-add
  double vs0 = 0.0, vs1 = 0.0, vs2 = 0.0;
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    vs0 = fma(0.125, vu[l], vs0);
    vs1 = fma(0.125, vv[l], vs1);
    vs2 = fma(0.125, vw[l], vs2);
  }
  // MARS impedances (:176-255)
  double mu[8];
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  const double q1c = qa * sspd;
#pragma unroll
  for (int l = 0; l < 8; ++l) {
    const double d0 = vu[l] - vs0, d1 = vv[l] - vs1, d2 = vw[l] - vs2;
    const double mag_vel = mode_sqrt(d0 * d0 + d1 * d1 + d2 * d2);
    const double muc = den * (q1c + qb * mag_vel);
    const double b0 = a.bmat[(size_t)(l * 3 + 0) * ne + e];
    const double b1 = a.bmat[(size_t)(l * 3 + 1) * ne + e];
    const double b2 = a.bmat[(size_t)(l * 3 + 2) * ne + e];
    const double mu_term = muc * mode_sqrt(b0 * b0 + b1 * b1 + b2 * b2);
    // the Riemann velocity's sums stay separately rounded in both modes: the
    // force's (v* - v) and then the element power cancel, and a contracted v*
    // would move a cold element's energy by ~1e-12 relative after one cycle
    s0 = FX_ADD(s0, FX_MUL(mu_term, vu[l]));
    s1 = FX_ADD(s1, FX_MUL(mu_term, vv[l]));
    s2 = FX_ADD(s2, FX_MUL(mu_term, vw[l]));
    s3 = s3 + mu_term;
    mu[l] = mu_term;
  }
  double vstar0 = 0.0, vstar1 = 0.0, vstar2 = 0.0;
  if (BR == 2 ? (br & FIERRO_BR_VSTAR) != 0 : s3 > a.fuzz) {
#if FIERRO_FMA
    const double rs3 = mode_rcp(s3);  // one reciprocal for the three components
    vstar0 = s0 * rs3;
    vstar1 = s1 * rs3;
    vstar2 = s2 * rs3;
#else
    const Divisor ds3 = divisor(s3);  // three correctly rounded quotients, one reciprocal seed
    vstar0 = quot(s0, ds3);
    vstar1 = quot(s1, ds3);
    vstar2 = quot(s2, ds3);
#endif
  }
  // shock detector (:287-315): r_face = 0.9 (div_nb + small) / (div + small) is
  // monotone in div_nb (non-decreasing for div + small > 0, non-increasing for < 0),
  // so the minimum over neighbours is attained at the smallest (resp. largest)
  // neighbour divergence and needs one division instead of one per neighbour.
  const double small = a.small;
  const double D = div + small;
  const int k0 = a.eie_start[e], k1 = a.eie_start[e + 1];
  long long kmin = 0x7FFFFFFFFFFFFFFFLL, kmax = (long long)0x8000000000000000ULL;
  for (int k = k0; k < k1; ++k) {
    const long long key = okey(__ldg(a.div + __ldg(a.eie + k)));
    kmin = key < kmin ? key : kmin;
    kmax = key > kmax ? key : kmax;
  }
  double r_min = 1.0;
  if (k1 > k0) {
    const double dsel = okey_decode(D > 0 ? kmin : kmax);
    const bool regular = isfinite(D) && D != 0.0 && isfinite(dsel);
    if (regular) {
      const double r_face = mode_div(0.9 * (dsel + small), D);
      r_min = okey(r_face) < okey(1.0) ? r_face : 1.0;
    } else {
      for (int k = k0; k < k1; ++k) {
        const double r_face = mode_div(0.9 * (__ldg(a.div + __ldg(a.eie + k)) + small), D);
        r_min = fmin(r_face, r_min);
      }
    }
  }
  double phi = 1.0 - fmax(0.0, r_min);  // pow(phi, 1.0) == phi
  // Mach-number detector (:318-328)
  const double c_length = pow_third(vol);
  // |div|: on the frozen trajectory, the sign recorded with the compression bit
  const double adiv = BR == 2 ? (compress ? -div : div) : fabs(div);
  const double araw = mode_div(20.0 * (c_length * adiv), sspd + a.fuzz);
  const double alpha = BR == 2 ? ((br & FIERRO_BR_MACH_CLAMP) ? 1.0 : araw) : fmin(1.0, araw);
  if (BR == 1) {
    // the limiter's case, and the neighbour that set r_min on the r_face branch
    unsigned lim = FIERRO_LIM_NONE;
    int sel = -1;
    const bool regular = isfinite(D) && D != 0.0 && isfinite(okey_decode(D > 0 ? kmin : kmax));
    if (k1 > k0 && !regular) {
      lim = FIERRO_LIM_IRREGULAR;
    } else if (r_min < 1.0 && r_min > 0.0) {
      lim = FIERRO_LIM_FACE;
      const long long ksel = D > 0 ? kmin : kmax;
      for (int k = k0; k < k1; ++k) {
        const int nb = __ldg(a.eie + k);
        if (okey(__ldg(a.div + nb)) == ksel) {
          sel = nb;
          break;
        }
      }
    } else if (!(r_min > 0.0)) {
      lim = FIERRO_LIM_FULL;
    }
    a.br_flags[e] = (unsigned char)((compress ? FIERRO_BR_COMPRESS : 0u) | (s3 > a.fuzz ? FIERRO_BR_VSTAR : 0u) |
                                    (araw < 1.0 ? 0u : FIERRO_BR_MACH_CLAMP) | (lim << FIERRO_BR_LIM_SHIFT));
    a.br_sel[e] = sel;
  }
  if (BR == 2) {
    const unsigned lim = (br >> FIERRO_BR_LIM_SHIFT) & 3u;
    if (lim == FIERRO_LIM_NONE) {
      phi = 0.0;
    } else if (lim == FIERRO_LIM_FULL) {
      phi = 1.0;
    } else if (lim == FIERRO_LIM_FACE && a.br_sel[e] >= 0) {
      phi = 1.0 - mode_div(0.9 * (__ldg(a.div + a.br_sel[e]) + small), D);
    }  // FIERRO_LIM_IRREGULAR: as evaluated above
  }
  if (TAPE) {
    double* t = a.tape + e;
#pragma unroll
    for (int l = 0; l < 8; ++l) {
      const double d0 = vu[l] - vs0, d1 = vv[l] - vs1, d2 = vw[l] - vs2;
      t[(size_t)l * ne] = mu[l];
      t[(size_t)(8 + l) * ne] = mode_sqrt(d0 * d0 + d1 * d1 + d2 * d2);
    }
    t[(size_t)16 * ne] = vstar0;
    t[(size_t)17 * ne] = vstar1;
    t[(size_t)18 * ne] = vstar2;
    t[(size_t)19 * ne] = s3;
    t[(size_t)20 * ne] = phi;
    t[(size_t)21 * ne] = araw;
    t[(size_t)22 * ne] = c_length;
    t[(size_t)23 * ne] = r_min;
    // the neighbour whose divergence set phi0 when the limiter is active
    int sel = -1;
    const long long ksel = D > 0 ? kmin : kmax;
    if (k1 > k0 && isfinite(D) && D != 0.0 && isfinite(okey_decode(ksel)) && r_min < 1.0 && r_min > 0.0) {
      for (int k = k0; k < k1; ++k) {
        const int nb = __ldg(a.eie + k);
        if (okey(__ldg(a.div + nb)) == ksel) {
          sel = nb;
          break;
        }
      }
    }
    a.tape_sel[e] = sel;
  }
  phi = alpha * phi;
  if (!STRENGTH) {
    // corner forces (:338-359)
#pragma unroll
    for (int l = 0; l < 8; ++l) {
      const double pm = phi * mu[l];
      const double b0 = a.bmat[(size_t)(l * 3 + 0) * ne + e];
      const double b1 = a.bmat[(size_t)(l * 3 + 1) * ne + e];
      const double b2 = a.bmat[(size_t)(l * 3 + 2) * ne + e];
      a.force[(size_t)(l * 3 + 0) * ne + e] = b0 * pres + pm * (vstar0 - vu[l]);
      a.force[(size_t)(l * 3 + 1) * ne + e] = b1 * pres + pm * (vstar1 - vv[l]);
      a.force[(size_t)(l * 3 + 2) * ne + e] = b2 * pres + pm * (vstar2 - vw[l]);
    }
  } else {
    // Cauchy stress tau = stress(1) - p I (:128-140), then the corner forces with
    // the inward normals -B (:98-102, :338-359)
    double sc[9], tau[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      sc[k] = a.stress_cur[(size_t)k * ne + e];
      tau[k] = sc[k];
    }
    tau[0] -= pres;
    tau[4] -= pres;
    tau[8] -= pres;
    const double vs[3] = {vstar0, vstar1, vstar2};
#pragma unroll
    for (int l = 0; l < 8; ++l) {
      const double pm = phi * mu[l];
      const double a0 = -a.bmat[(size_t)(l * 3 + 0) * ne + e];
      const double a1 = -a.bmat[(size_t)(l * 3 + 1) * ne + e];
      const double a2 = -a.bmat[(size_t)(l * 3 + 2) * ne + e];
      const double vl[3] = {vu[l], vv[l], vw[l]};
#pragma unroll
      for (int d = 0; d < 3; ++d)
        a.force[(size_t)(l * 3 + d) * ne + e] =
            a0 * tau[d] + a1 * tau[3 + d] + a2 * tau[6 + d] + pm * (vs[d] - vl[d]);
    }
    // stress update of hypo materials (:362-391); the others carry stress(1) over
    // from the cycle-start bin on the first stage (rk_init's copy)
    if (a.stype[mat] == 1) {
      double L[9], s0[9];
      velocity_gradient(vu, vv, vw, a.bmat, ne, e, vol, L);
#pragma unroll
      for (int k = 0; k < 9; ++k) s0[k] = a.stress0[(size_t)k * ne + e];
      user_strength_model(sc, s0, L, a.statev + e, ne, mat, den, a.sie0[e], vol, a.ctrl->dt, a.rk_alpha);
#pragma unroll
      for (int k = 0; k < 9; ++k) a.stress_out[(size_t)k * ne + e] = sc[k];
    } else if (a.copy_stress) {
#pragma unroll
      for (int k = 0; k < 9; ++k) a.stress_out[(size_t)k * ne + e] = sc[k];
    }
  }
}

// One thread per element; a batch may run as a persistent grid (a.grid blocks)
// that strides over the elements.
template <bool BATCH, bool TAPE, bool STRENGTH, int BR = 0>
__global__ void FIERRO_FORCE_BOUNDS k_force(const ForceArgs a) {
  if (BATCH) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < a.ne; e += gridDim.x * blockDim.x)
      force_elem<true, TAPE, STRENGTH, BR>(a, e);
  } else {
    if (!a.ctrl->active) return;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= a.ne) return;
    force_elem<false, TAPE, STRENGTH, BR>(a, e);
  }
}

// ---------------------------------------------------------------------------
// Node update: corner-force gather in the reference's summation order, velocity,
// boundary conditions, half velocity and position.
template <bool BATCH, bool COH = false>
__device__ __forceinline__ void node_update(const NodeArgs& a, const int n) {
  const Ctrl* ctrl = BATCH ? a.ctrl + a.inst[n] : a.ctrl;
  if (BATCH && !ctrl->active) return;
  const size_t ne = (size_t)a.ne;
  double f0 = 0.0, f1 = 0.0, f2 = 0.0;
  const int c0 = a.cin_start[n], c1 = a.cin_start[n + 1];
  // corners kNodeGather at a time: the corner ids, then their force loads, are
  // issued before the sums, which keep the corner order
  for (int base = c0; base < c1; base += kNodeGather) {
    const int cnt = min(kNodeGather, c1 - base);
    int cid[kNodeGather];
#pragma unroll
    for (int k = 0; k < kNodeGather; ++k) cid[k] = k < cnt ? __ldg(a.cin + base + k) : 0;
    double g[kNodeGather][3];
#pragma unroll
    for (int k = 0; k < kNodeGather; ++k) {
      const int e = cid[k] >> 3, l = cid[k] & 7;
#pragma unroll
      for (int d = 0; d < 3; ++d) g[k][d] = k < cnt ? ld_ro<COH>(a.force + (size_t)(l * 3 + d) * ne + e) : 0.0;
    }
#pragma unroll
    for (int k = 0; k < kNodeGather; ++k)
      if (k < cnt) {
        f0 = f0 + g[k][0];
        f1 = f1 + g[k][1];
        f2 = f2 + g[k][2];
      }
  }
  const double adt = a.rk_alpha * ctrl->dt;
  const double u0 = a.u0[n], v0 = a.v0[n], w0 = a.w0[n];
#if FIERRO_FMA
  // the reciprocal of the node's mass, formed once per uploaded state (the
  // same IEEE division, so the same bits as forming it here every stage)
  const double rm = a.node_rm ? a.node_rm[n] : 1.0 / a.node_mass[n];
  double u1 = u0 + adt * f0 * rm;
  double v1 = v0 + adt * f1 * rm;
  double w1 = w0 + adt * f2 * rm;
#else
  const Divisor m = divisor(a.node_mass[n]);  // correctly rounded quotients, one reciprocal seed
  double u1 = u0 + quot(adt * f0, m);
  double v1 = v0 + quot(adt * f1, m);
  double w1 = w0 + quot(adt * f2, m);
#endif
  const unsigned bc = a.bc_mask[n];
  if (bc & 1u) u1 = 0.0;
  if (bc & 2u) v1 = 0.0;
  if (bc & 4u) w1 = 0.0;
  const double hu = (u1 + u0) * 0.5, hv = (v1 + v0) * 0.5, hw = (w1 + w0) * 0.5;
  a.u1[n] = u1;
  a.v1[n] = v1;
  a.w1[n] = w1;
  a.hx[n] = hu;
  a.hy[n] = hv;
  a.hz[n] = hw;
  a.x1[n] = a.x0[n] + adt * hu;
  a.y1[n] = a.y0[n] + adt * hv;
  a.z1[n] = a.z0[n] + adt * hw;
}

// One thread per node; a batch may run as a persistent grid striding over the nodes.
template <bool BATCH>
__global__ void __launch_bounds__(kNodeBlock) k_node(const NodeArgs a) {
  if (BATCH) {
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < a.nn; n += gridDim.x * blockDim.x)
      node_update<true>(a, n);
  } else {
    if (!a.ctrl->active) return;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.nn) return;
    node_update<false>(a, n);
  }
}

// ---------------------------------------------------------------------------
// Element update.  KIND 0: stage; 1: last stage (adds the CFL partials);
// 2: prime (corner normals, divergence and CFL of an uploaded state).
// STRENGTH (a handle with a hyper material) runs the hyper model between the
// density and the EOS (properties.cpp:46-95) with the velocity gradient of the
// updated state.
// A tile is one block's worth of elements, with one CFL partial.  In a batch
// every tile lies inside one instance (instances' element ranges are padded to
// whole default blocks, padding marked by a negative instance id, and the block
// divides the default), so the activity test and the CFL partial are per tile.
template <int KIND, bool BATCH, bool STRENGTH, bool COH = false>
__device__ __forceinline__ void elem_tile(const ElemArgs& a, const int tile) {
  const int e = tile * blockDim.x + threadIdx.x;
  const int ib = BATCH ? a.inst[tile * blockDim.x] : 0;
  Ctrl* ctrl = a.ctrl + ib;
  if (KIND != 2 && !ctrl->active) return;
  const bool live = e < a.ne && (!BATCH || a.inst[e] >= 0);
  const double dt_cfl = BATCH ? a.dt_cfl_tab[ib] : a.dt_cfl;
  long long dkey = 0x7FFFFFFFFFFFFFFFLL;
  if (live) {
    const int ne = a.ne;
    const int4 n03 = __ldg(reinterpret_cast<const int4*>(a.nie) + 2 * e);
    const int4 n47 = __ldg(reinterpret_cast<const int4*>(a.nie) + 2 * e + 1);
    const int nid[8] = {n03.x, n03.y, n03.z, n03.w, n47.x, n47.y, n47.z, n47.w};
    double x[8], y[8], z[8], u[8], v[8], w[8];
#pragma unroll
    for (int l = 0; l < 8; ++l) {
      x[l] = ld_ro<COH>(a.x + nid[l]);
      y[l] = ld_ro<COH>(a.y + nid[l]);
      z[l] = ld_ro<COH>(a.z + nid[l]);
      u[l] = ld_ro<COH>(a.u + nid[l]);
      v[l] = ld_ro<COH>(a.v + nid[l]);
      w[l] = ld_ro<COH>(a.w + nid[l]);
    }
    double sie1 = 0.0;
    if (KIND != 2) {
      // energy (energy_sgh.cpp:16-52): power = sum_c F_c . (v1 + v0)/2, lid-major,
      // separately rounded in both modes: where a cold element's heating nearly
      // cancels its energy, a contracted sum would move sie by far more than an ulp
      double power = 0.0;
#pragma unroll
      for (int l = 0; l < 8; ++l) {
        power = FX_ADD(power, FX_MUL(ld_pl<COH>(a.force + (size_t)(l * 3 + 0) * ne + e), ld_ro<COH>(a.hx + nid[l])));
        power = FX_ADD(power, FX_MUL(ld_pl<COH>(a.force + (size_t)(l * 3 + 1) * ne + e), ld_ro<COH>(a.hy + nid[l])));
        power = FX_ADD(power, FX_MUL(ld_pl<COH>(a.force + (size_t)(l * 3 + 2) * ne + e), ld_ro<COH>(a.hz + nid[l])));
      }
      const double adt = a.rk_alpha * ctrl->dt;
      sie1 = a.sie0[e] - FX_MUL(mode_div(adt, a.mass[e]), power);  // not fused: sie1 may cancel sie0
      a.sie1[e] = sie1;
    }
    double vol_geo, Sx, Sy, Sz;
    hex_geometry(x, y, z, u, v, w, a.bmat, ne, e, vol_geo, Sx, Sy, Sz);
    // the priming pass keeps the uploaded volume, as get_divergence reads elem_vol
    const double vol = (KIND == 2) ? a.vol[e] : vol_geo;
    // divergence for the next stage (momentum.cpp:265-286), with this geometry
    const double inverse_vol = mode_rcp(vol);
    double div = 0.0;
    div = div + Sx * inverse_vol;
    div = div + Sy * inverse_vol;
    div = div + Sz * inverse_vol;
    a.div[e] = div;
    double sspd;
    if (KIND != 2) {
      a.vol[e] = vol;
      // update_state (properties.cpp:39, 98-109; ideal_gas eos.cpp:35-43)
      const double den = mode_div(a.mass[e], vol);
      if (STRENGTH) {
        const int mat = a.mat[e];
        if (a.stype[mat] == 2) {
          double L[9], s0[9], s1[9];
          velocity_gradient(u, v, w, a.bmat, ne, e, vol, L);
#pragma unroll
          for (int k = 0; k < 9; ++k) {
            s0[k] = a.stress0[(size_t)k * ne + e];
            s1[k] = a.stress1[(size_t)k * ne + e];
          }
          user_strength_model(s1, s0, L, a.statev + e, ne, mat, den, a.sie0[e], vol, ctrl->dt, a.rk_alpha);
#pragma unroll
          for (int k = 0; k < 9; ++k) a.stress1[(size_t)k * ne + e] = s1[k];
        }
      }
      const double gamma = a.gamma[e], csmin = a.csmin[e];
      const double pres = (gamma - 1.0) * sie1 * den;
      sspd = mode_sqrt(gamma * (gamma - 1.0) * sie1);
      if (sspd < csmin) sspd = csmin;
      a.den[e] = den;
      a.pres[e] = pres;
      a.sspd[e] = sspd;
      if (!(vol > 0.0) || !isfinite(vol)) atomicOr(&ctrl->status, FIERRO_STATUS_BAD_VOLUME);
      if (!isfinite(sie1) || !isfinite(pres)) atomicOr(&ctrl->status, FIERRO_STATUS_BAD_STATE);
    } else {
      sspd = a.sspd[e];
    }
    if (KIND != 0) {
      // element CFL step dt_cfl * min distance / (c + fuzz) (time_integration.cpp:124-131);
      // min of the square roots == square root of the min (sqrt is monotone, exact).
      // The coordinates go to this thread's column of shared memory for the exact
      // re-evaluation of the screened pairs (no other thread reads them).
      __shared__ double s_xyz[24][kElemBlock];
#pragma unroll
      for (int l = 0; l < 8; ++l) {
        s_xyz[l][threadIdx.x] = x[l];
        s_xyz[8 + l][threadIdx.x] = y[l];
        s_xyz[16 + l][threadIdx.x] = z[l];
      }
      const double d2min = cfl::min_d2(x, y, z, &s_xyz[0][threadIdx.x], &s_xyz[8][threadIdx.x],
                                       &s_xyz[16][threadIdx.x], kElemBlock);
      const double dist_min = mode_sqrt(d2min);
      const double dt_l = mode_div(dt_cfl * dist_min, sspd + a.fuzz);
      dkey = isnan(dt_l) ? 0x7FFFFFFFFFFFFFFFLL : okey(dt_l);
    }
  }
  if (KIND != 0) {
    const long long k = block_min_key(dkey);
    if (threadIdx.x == 0) a.cfl_part[tile] = k;
  }
}

// One tile per block; a batch may run as a persistent grid looping over the
// tiles (a barrier between tiles, as the CFL reduction reuses shared memory).
template <int KIND, bool BATCH, bool STRENGTH>
__global__ void FIERRO_ELEM_BOUNDS k_elem(const ElemArgs a) {
  if (BATCH) {
    const int ntiles = (a.ne + blockDim.x - 1) / blockDim.x;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      elem_tile<KIND, true, STRENGTH>(a, t);
      __syncthreads();
    }
  } else {
    elem_tile<KIND, false, STRENGTH>(a, blockIdx.x);
  }
}

// ---------------------------------------------------------------------------
// A batch's RK stage in one cooperative launch: the force pass, a grid barrier,
// the node pass, a grid barrier, the element pass, each over the whole batch
// with the grid's resident blocks striding over elements, nodes and element
// tiles (the same device functions as the three separate kernels, so the same
// results bit for bit).  Values an earlier phase wrote are read from L2 (COH).
// Every wait at a barrier has an iteration limit: a block that gives up sets
// FIERRO_SYNC_TIMEOUT and returns, and so does every other block at its own
// limit, so a launch always ends.
constexpr unsigned kSyncSpins = 1u << 23;  // x ~128 ns: about a second

__device__ __forceinline__ bool grid_barrier(const StageSync& s) {
  __shared__ unsigned ok_s;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned ok = 1u;
    volatile unsigned* gen = s.gen;
    const unsigned g = *gen;
    if (atomicAdd(s.arrive, 1u) == gridDim.x - 1) {
      atomicExch(s.arrive, 0u);
      __threadfence();
      atomicAdd(s.gen, 1u);
    } else {
      for (unsigned it = 0; *gen == g; ++it) {
        if (it > kSyncSpins) {
          atomicOr(s.status, FIERRO_SYNC_TIMEOUT);
          ok = 0u;
          break;
        }
        __nanosleep(128);
      }
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0u;
}

template <int KIND>
__global__ void __launch_bounds__(kElemBlock) k_stage_fused(const ForceArgs fa, const NodeArgs na, const ElemArgs ea,
                                                            const StageSync sync) {
  const int stride = gridDim.x * blockDim.x;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < fa.ne; e += stride) force_elem<true, false, false, 0>(fa, e);
  if (!grid_barrier(sync)) return;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < na.nn; n += stride) node_update<true, true>(na, n);
  if (!grid_barrier(sync)) return;
  const int ntiles = (ea.ne + blockDim.x - 1) / blockDim.x;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    elem_tile<KIND, true, false, true>(ea, t);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// get_timestep's scalar part (time_integration.cpp:69-150) on the device.  The
// per-element clamp to [dt_min, dt_max] commutes with the minimum (it is
// monotone), so it is applied once to the minimum.
__device__ __forceinline__ void dt_update(Ctrl* c, long long k, const LoopParams& lp) {
  if (c->stopped) {
    c->active = 0;
    return;
  }
  double dt = c->dt * 1.1;
  double min_dt_calc = (k == 0x7FFFFFFFFFFFFFFFLL) ? 1.7976931348623157e308 : okey_decode(k);
  if (min_dt_calc < lp.dt_min) c->status |= FIERRO_STATUS_DT_FLOOR;
  min_dt_calc = fmin(min_dt_calc, lp.dt_max);
  min_dt_calc = fmax(min_dt_calc, lp.dt_min);
  if (min_dt_calc < dt) dt = min_dt_calc;
  dt = fmin(dt, (c->graphics_time - c->time_value) + lp.fuzz);
  dt = fmin(dt, lp.time_final - c->time_value);
  c->dt = dt;
  c->active = 1;
}

__global__ void __launch_bounds__(1024) k_dt(const DtArgs a) {
  long long k = 0x7FFFFFFFFFFFFFFFLL;
  for (int i = threadIdx.x; i < a.nparts; i += blockDim.x) {
    const long long t = a.cfl_part[i];
    k = t < k ? t : k;
  }
  k = block_min_key(k);
  if (threadIdx.x == 0) dt_update(a.ctrl, k, a.lp);
}

// One block per instance: instance i's CFL partials are cfl_part[part_start[i] ..
// part_start[i+1]).
__global__ void __launch_bounds__(256) k_dt_batch(const DtArgs a) {
  const int i = blockIdx.x;
  long long k = 0x7FFFFFFFFFFFFFFFLL;
  for (int j = a.part_start[i] + threadIdx.x; j < a.part_start[i + 1]; j += blockDim.x) {
    const long long t = a.cfl_part[j];
    k = t < k ? t : k;
  }
  k = block_min_key(k);
  if (threadIdx.x == 0) dt_update(a.ctrl + i, k, a.lps[i]);
}

// End of a cycle (sgh_solve.cpp:590-632).
__device__ __forceinline__ void end_update(Ctrl* c, const LoopParams& lp) {
  c->wrote = 0;
  if (!c->active) return;
  c->time_value += c->dt;
  const long long cycle = c->cycle;
  bool write = false;
  if ((cycle + 1) % lp.graphics_cyc_ival == 0 && cycle > 0) write = true;
  else if (c->time_value >= lp.time_final) write = true;
  else if (c->time_value >= c->graphics_time) write = true;
  if (write) c->graphics_time = c->time_value + lp.graphics_dt_ival;
  c->wrote = write ? 1 : 0;
  if (c->time_value >= lp.time_final) c->stopped = 1;
  c->cycle = cycle + 1;
  c->active = 0;
}

__global__ void k_end(Ctrl* c, const LoopParams lp) { end_update(c, lp); }

__global__ void k_end_batch(Ctrl* c, const LoopParams* lps, int ninst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ninst) end_update(c + i, lps[i]);
}

// Energy tallies (sgh_solve.cpp:77-101): fixed-shape two-pass sums.
__global__ void __launch_bounds__(kEnergyBlock) k_energy_part(const EnergyArgs a) {
  __shared__ double sh[2][kEnergyBlock];
  double ie = 0.0, ke = 0.0;
  const int stride = gridDim.x * blockDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.ne; i += stride) ie += a.mass[i] * a.sie[i];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nn; i += stride) {
    double k = 0;
    k += a.u[i] * a.u[i];
    k += a.v[i] * a.v[i];
    k += a.w[i] * a.w[i];
    ke += a.node_mass[i] * k;
  }
  sh[0][threadIdx.x] = ie;
  sh[1][threadIdx.x] = ke;
  __syncthreads();
  for (int s = kEnergyBlock / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + s];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    a.part[blockIdx.x] = sh[0][0];
    a.part[gridDim.x + blockIdx.x] = sh[1][0];
  }
}

__global__ void k_energy_final(const EnergyArgs a, int nblocks) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double ie = 0.0, ke = 0.0;
  for (int b = 0; b < nblocks; ++b) {
    ie += a.part[b];
    ke += a.part[nblocks + b];
  }
  a.out[0] = ie;
  a.out[1] = 0.5 * ke;
}

// ---------------------------------------------------------------------------
static unsigned blocks_for(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// A block size below the default only lowers the threads per block (the
// kernels' shared memory is sized for the default); a batch keeps the default,
// as its instances' element ranges are padded to whole default blocks.
static int block_or(int b, int def) { return (b >= 32 && b <= def && b % 32 == 0) ? b : def; }

// A batch's persistent grid (a.grid > 0 blocks) never exceeds one block per tile.
static unsigned grid_or(int grid, unsigned blocks) {
  return (grid > 0 && (unsigned)grid < blocks) ? (unsigned)grid : blocks;
}

static void launch_force(const ForceArgs& a, cudaStream_t s) {
  const int bs = block_or(a.block, kForceBlock);
  const unsigned g = blocks_for(a.ne, bs);
  if (a.inst) k_force<true, false, false><<<grid_or(a.grid, g), bs, 0, s>>>(a);
  else if (a.stress_out) k_force<false, false, true><<<g, bs, 0, s>>>(a);
  else k_force<false, false, false><<<g, bs, 0, s>>>(a);
}
static void launch_force_tape(const ForceArgs& a, cudaStream_t s) {
  const int bs = block_or(a.block, kForceBlock);
  k_force<false, true, false><<<blocks_for(a.ne, bs), bs, 0, s>>>(a);
}
static void launch_force_branch(const ForceArgs& a, int mode, cudaStream_t s) {
  const int bs = block_or(a.block, kForceBlock);
  if (mode == 1) k_force<false, false, false, 1><<<blocks_for(a.ne, bs), bs, 0, s>>>(a);
  else k_force<false, false, false, 2><<<blocks_for(a.ne, bs), bs, 0, s>>>(a);
}
static void launch_node(const NodeArgs& a, cudaStream_t s) {
  const int bs = block_or(a.block, kNodeBlock);
  if (a.inst) k_node<true><<<grid_or(a.grid, blocks_for(a.nn, bs)), bs, 0, s>>>(a);
  else k_node<false><<<blocks_for(a.nn, bs), bs, 0, s>>>(a);
}
template <bool B, bool S>
static void launch_elem_t(const ElemArgs& a, int kind, cudaStream_t s) {
  const int bs = block_or(a.block, kElemBlock);
  const unsigned g = B ? grid_or(a.grid, blocks_for(a.ne, bs)) : blocks_for(a.ne, bs);
  if (kind == 0) k_elem<0, B, S><<<g, bs, 0, s>>>(a);
  else if (kind == 1) k_elem<1, B, S><<<g, bs, 0, s>>>(a);
  else k_elem<2, B, false><<<g, bs, 0, s>>>(a);
}
static void launch_elem(const ElemArgs& a, int kind, cudaStream_t s) {
  if (a.inst) launch_elem_t<true, false>(a, kind, s);
  else if (a.stress1) launch_elem_t<false, true>(a, kind, s);
  else launch_elem_t<false, false>(a, kind, s);
}
static void launch_dt(const DtArgs& a, cudaStream_t s) {
  if (a.part_start) k_dt_batch<<<a.ninst, 256, 0, s>>>(a);
  else k_dt<<<1, 1024, 0, s>>>(a);
}
static void launch_end(Ctrl* c, const LoopParams& lp, cudaStream_t s) { k_end<<<1, 1, 0, s>>>(c, lp); }
static void launch_end_batch(Ctrl* c, const LoopParams* lps, int ninst, cudaStream_t s) {
  k_end_batch<<<blocks_for(ninst, 128), 128, 0, s>>>(c, lps, ninst);
}
static int batch_max_blocks(int kernel, int block) {
  int n = 0;
  cudaError_t err = cudaSuccess;
  if (kernel == 0) err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_force<true, false, false>, block, 0);
  else if (kernel == 1) err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_node<true>, block, 0);
  else err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_elem<1, true, false>, block, 0);
  return err == cudaSuccess && n > 0 ? n : 1;
}
__global__ void k_reciprocal(const double* __restrict__ in, double* __restrict__ out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = 1.0 / in[i];
}
static void launch_reciprocal(const double* in, double* out, int n, cudaStream_t s) {
  if (n > 0) k_reciprocal<<<blocks_for(n, 256), 256, 0, s>>>(in, out, n);
}
// The mode's square and cube roots, quotients and reciprocals (mode_sqrt,
// mode_cbrt, quot, mode_rcp) against the library's on n inputs.  which 0..3:
// eight special values (zero, -0, the smallest subnormal, infinity, NaN, -1, the
// largest and the smallest normal double), then seeded 2^E (1 + f) with E
// uniform in [lo_exp, hi_exp] and f's 52 bits uniform (quotients: two such
// operands of random signs, the special value as the divisor, signed zeros as
// the dividend of the next eight).  which 4..6: the
// square root, quotient and reciprocal on arguments whose exact result lies
// within 2^-55 .. 2^-13 of an ulp of a rounding boundary (scaled by random
// powers of two): 4^s (1 + (2k+1) 2^-52) and 4^s (1 - (2k+1) 2^-53), whose
// square roots lie just below the midpoints 4^s/2^s (1 + (2k+1) 2^-53) and
// 2^s (1 - (2k+1) 2^-54); 2^s (1 - (2k+1) 2^-53), whose reciprocal lies just
// above the midpoint 2^-s (1 + (2k+1) 2^-53); and 2^t (1 + m 2^-52) / that,
// just above a midpoint too (k < 2^20, m < 2^16).  which 7, 8: the adjoint's
// ~2^-43 reciprocal and reciprocal square root (fast_rcp, fast_rsqrt) against
// 1 / x and 1 / sqrt(x), on the seeded arguments.  out[0] counts results
// differing, out[1] is the largest difference in ulps, out[2] counts results
// differing by more than one ulp.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double seeded_double(unsigned long long h, int lo_exp, int hi_exp, bool sign) {
  const int E = lo_exp + (int)((h >> 40) % (unsigned long long)(hi_exp - lo_exp + 1));
  const long long s = sign ? (long long)((mix64(h ^ 0x5555ULL) >> 63) << 63) : 0LL;
  return __longlong_as_double(s | ((long long)(E + 1023) << 52) | (long long)(mix64(h) & 0xFFFFFFFFFFFFFULL));
}
__global__ void __launch_bounds__(256) k_root_check(int which, long long n, unsigned long long seed, int lo_exp,
                                                    int hi_exp, unsigned long long* out) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) {
    const unsigned long long h = mix64(seed ^ (unsigned long long)i * 0xD1B54A32D192ED03ULL);
    const long long odd = 2 * (long long)((unsigned long long)i & 0xFFFFF) + 1;  // 2k + 1, k < 2^20
    const int s = (int)((h >> 40) % 201) - 100;                                  // a power of two in +-100
    double x;
    if (which >= 4 && which <= 6) {
      if (which == 4)
        x = __longlong_as_double((i & 1) ? ((long long)(1023 + 2 * s) << 52) - odd
                                         : ((long long)(1023 + 2 * s) << 52) | odd);
      else
        x = __longlong_as_double(((long long)(1023 + s) << 52) - odd);
    } else if (i < 8) {
      const long long special[8] = {0LL, (long long)0x8000000000000000ULL, 1LL, 0x7FF0000000000000LL,
                                    0x7FF8000000000000LL, (long long)0xBFF0000000000000ULL, 0x7FEFFFFFFFFFFFFFLL,
                                    0x0010000000000000LL};
      x = __longlong_as_double(special[i]);
    } else {
      x = seeded_double(h, lo_exp, hi_exp, which == 2 || which == 3 || which == 7);
    }
    double a, r;
    if (which == 0 || which == 4) {
      a = mode_sqrt(x);
      r = sqrt(x);
    } else if (which == 1) {
      a = mode_cbrt(x);
      r = cbrt(x);
    } else if (which == 2 || which == 5) {
      const int t = (int)((mix64(h + 7) >> 40) % 201) - 100;
      double num = which == 2 ? seeded_double(mix64(h + 1), lo_exp, hi_exp, true)
                              : __longlong_as_double(((long long)(1023 + t) << 52) | (long long)(h & 0xFFFF));
      if (which == 2 && i >= 8 && i < 16) num = (i & 1) ? -0.0 : 0.0;  // signed zeros over seeded divisors
      a = quot(num, divisor(x));  // the shared-divisor form (mode_div in the FMA mode)
      r = num / x;
    } else if (which == 3 || which == 6) {
      a = mode_rcp(x);
      r = 1.0 / x;
    } else if (which == 7) {
      a = fast_rcp(x);
      r = 1.0 / x;
    } else {
      a = fast_rsqrt(x);
      r = 1.0 / sqrt(x);
    }
    long long d = __double_as_longlong(a) - __double_as_longlong(r);
    if (isnan(a) && isnan(r)) d = 0;
    if (d < 0) d = -d;
    if (d) {
      atomicAdd(out, 1ULL);
      atomicMax(out + 1, (unsigned long long)d);
      if (d > 1) atomicAdd(out + 2, 1ULL);
    }
  }
}
static void launch_root_check(int which, long long n, unsigned long long seed, int lo_exp, int hi_exp,
                              unsigned long long* out, cudaStream_t s) {
  const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 16);
  k_root_check<<<(unsigned)blocks, 256, 0, s>>>(which, n, seed, lo_exp, hi_exp, out);
}
static cudaError_t launch_stage_fused(const ForceArgs& fa, const NodeArgs& na, const ElemArgs& ea, int kind,
                                      const StageSync& sync, int grid, int cooperative, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block_or(ea.block, kElemBlock));
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = cooperative ? 1 : 0;
  return kind == 1 ? cudaLaunchKernelEx(&cfg, k_stage_fused<1>, fa, na, ea, sync)
                   : cudaLaunchKernelEx(&cfg, k_stage_fused<0>, fa, na, ea, sync);
}
static int fused_max_blocks(int block) {
  int n0 = 0, n1 = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n0, k_stage_fused<0>, block, 0) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n1, k_stage_fused<1>, block, 0) != cudaSuccess)
    return 0;
  return n0 < n1 ? n0 : n1;
}
static void launch_energy(const EnergyArgs& a, cudaStream_t s) {
  const int nb = 512;
  k_energy_part<<<nb, kEnergyBlock, 0, s>>>(a);
  k_energy_final<<<1, 32, 0, s>>>(a, nb);
}

}  // namespace FIERRO_IMPL

#if FIERRO_FMA
const KernelSet& kernels_fma() {
  static const KernelSet k = {fma_impl::launch_force, fma_impl::launch_force_tape, fma_impl::launch_force_branch, fma_impl::launch_node, fma_impl::launch_elem,
                              fma_impl::launch_dt, fma_impl::launch_end, fma_impl::launch_energy,
                              fma_impl::launch_end_batch, "fma", fma_impl::batch_max_blocks,
                              fma_impl::launch_reciprocal, fma_impl::launch_root_check,
                              fma_impl::launch_stage_fused, fma_impl::fused_max_blocks};
  return k;
}
#else
const KernelSet& kernels_exact() {
  static const KernelSet k = {exact_impl::launch_force, exact_impl::launch_force_tape, exact_impl::launch_force_branch, exact_impl::launch_node, exact_impl::launch_elem,
                              exact_impl::launch_dt, exact_impl::launch_end, exact_impl::launch_energy,
                              exact_impl::launch_end_batch, "exact", exact_impl::batch_max_blocks,
                              exact_impl::launch_reciprocal, exact_impl::launch_root_check,
                              exact_impl::launch_stage_fused, exact_impl::fused_max_blocks};
  return k;
}
#endif

}  // namespace fierro
