// 2D-RZ SGH kernels for sm_103a (GB300), FP64: the num_dims == 2 branches of
// Explicit-Lagrange-Kokkos/SGH_solver on quad meshes (x axial, y radial).
//
// Compiled twice, like sgh_kernels.cu: FIERRO_FMA=0 with --fmad=false (every
// operation the reference's, in its order; square roots and shared-divisor
// quotients by the correctly rounded Newton forms of sgh_common.cuh) and
// FIERRO_FMA=1 (contraction and reciprocal reuse allowed; the Newton square
// roots, quotients and reciprocals).
//
// One cycle is 2 + 4*rk_num_stages launches: k_dt, then per RK stage
//   k_force_rz (elements)  corner normals, area and Barlow corner areas of the
//                          stage's input quad, MARS forces with the hoop terms,
//                          hypo strength model (force_sgh.cpp:407-808)
//   k_node_rz  (nodes)     corner-force gather, velocity, boundary conditions,
//                          position, and the areal node mass of the new position
//                          (momentum.cpp:11-53, boundary.cpp:10-55,
//                          geometry.cpp:9-26, sgh_solve.cpp:496-505)
//   k_axis_rz  (boundary nodes) nodes on the axis take the largest half-mass of
//                          their off-axis edge neighbours (sgh_solve.cpp:547-578)
//   k_elem_rz  (elements)  radius-weighted energy (energy_sgh.cpp:6-55), RZ volume
//                          (geometry.cpp:369-434), density and EOS
//                          (properties.cpp:118-219), the next stage's divergence
//                          (momentum.cpp:298-378) and on the last stage the CFL
//                          step (time_integration.cpp:161-246)
// then k_end.  Nothing is accumulated with atomics.
#include <cstdint>

#include "sgh_rz.h"

#ifndef FIERRO_FMA
#error "compile with -DFIERRO_FMA=0 or -DFIERRO_FMA=1"
#endif

#if FIERRO_FMA
#define FIERRO_RZ_IMPL rz_fma_impl
#else
#define FIERRO_RZ_IMPL rz_exact_impl
#endif

namespace fierro {
namespace FIERRO_RZ_IMPL {

#include "sgh_common.cuh"
#include "sgh_user_mat.cuh"

constexpr int kRzBlock = 128;
constexpr int kRzNodeBlock = 256;

// get_bmatrix2D (geometry.cpp:315-365): outward corner normals B[l][dim].
__device__ __forceinline__ void rz_bmatrix(const double (&x)[4], const double (&y)[4], double (&B)[4][2]) {
  B[0][0] = -0.5 * (y[3] - y[1]);
  B[1][0] = -0.5 * (y[0] - y[2]);
  B[2][0] = -0.5 * (y[1] - y[3]);
  B[3][0] = -0.5 * (y[2] - y[0]);
  B[0][1] = -0.5 * (x[1] - x[3]);
  B[1][1] = -0.5 * (x[2] - x[0]);
  B[2][1] = -0.5 * (x[3] - x[1]);
  B[3][1] = -0.5 * (x[0] - x[2]);
}

// get_area_quad (geometry.cpp:438-466)
__device__ __forceinline__ double rz_area(const double (&x)[4], const double (&y)[4]) {
  return 0.5 * ((x[0] - x[2]) * (y[1] - y[3]) + (x[3] - x[1]) * (y[0] - y[2]));
}

// get_vol_quad (geometry.cpp:369-434): volume per radian of the revolved quad.
__device__ __forceinline__ double rz_vol(const double (&x)[4], const double (&y)[4]) {
  return ((y[2] + y[3] + y[0]) * ((y[2] - y[3]) * (x[0] - x[3]) - (y[0] - y[3]) * (x[2] - x[3])) +
          (y[0] + y[1] + y[2]) * ((y[0] - y[1]) * (x[2] - x[1]) - (y[2] - y[1]) * (x[0] - x[1]))) /
         6.0;
}

// heron (geometry.cpp:470-500)
__device__ __forceinline__ double rz_heron(double x1, double y1, double x2, double y2, double x3, double y3) {
  double S = 0.0;
  const double a = sqrt((x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1));
  S = S + a;
  const double b = sqrt((x3 - x2) * (x3 - x2) + (y3 - y2) * (y3 - y2));
  S = S + b;
  const double c = sqrt((x3 - x1) * (x3 - x1) + (y3 - y1) * (y3 - y1));
  S = S + c;
  S = S * 0.5;
  return sqrt(S * (S - a) * (S - b) * (S - c));
}

// get_area_weights2D (geometry.cpp:503-547): Barlow's corner areas.
__device__ __forceinline__ void rz_corner_areas(const double (&x)[4], const double (&y)[4], double (&ca)[4]) {
  double rc = 0.0, zc = 0.0;
#pragma unroll
  for (int l = 0; l < 4; ++l) {
    rc = rc + 0.25 * y[l];
    zc = zc + 0.25 * x[l];
  }
  const double A12 = rz_heron(x[0], y[0], zc, rc, x[1], y[1]);
  const double A23 = rz_heron(x[1], y[1], zc, rc, x[2], y[2]);
  const double A34 = rz_heron(x[2], y[2], zc, rc, x[3], y[3]);
  const double A41 = rz_heron(x[3], y[3], zc, rc, x[0], y[0]);
  ca[0] = (5. * A41 + 5. * A12 + A23 + A34) / 12.;
  ca[1] = (A41 + 5. * A12 + 5. * A23 + A34) / 12.;
  ca[2] = (A41 + A12 + 5. * A23 + 5. * A34) / 12.;
  ca[3] = (5. * A41 + A12 + A23 + 5. * A34) / 12.;
}

// Without stress the hoop terms are tau(1,0) A_c / r = (+0 A_c) / r and
// (tau(1,1) - tau(2,2)) A_c / r = ((0 - p) - (0 - p)) A_c / r: exactly +0.0
// whenever p and the corner area A_c are finite.  A_c is finite unless one of
// Heron's factors s - a, s - b, s - c of a centroid triangle rounds to zero or
// below.  For a triangle of area T and semi-perimeter s, each factor is at least
// T^2 / s^3 (the product of all three is T^2 / s and each is below s), while the
// computed factors carry an absolute error of about 9 eps s (sides and s to a few
// ulps each); so T > 3 sqrt(eps) s^2 ~ 3.2e-8 s^2 keeps every computed factor
// positive.  With s <= P / 2 for the L1 perimeter P, |cross| = 2T > 1e-4 P^2 is
// sufficient by more than three orders of magnitude, and its own rounding (a few
// eps P^2) does not matter.  True for all four centroid triangles (and NaN-free
// coordinates) means the corner areas need not be formed; otherwise they are,
// as the reference does.
__device__ __forceinline__ bool rz_corner_areas_finite(const double (&x)[4], const double (&y)[4]) {
  double rc = 0.0, zc = 0.0;
#pragma unroll
  for (int l = 0; l < 4; ++l) {
    rc = rc + 0.25 * y[l];
    zc = zc + 0.25 * x[l];
  }
  bool ok = true;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int j = (i + 1) & 3;
    const double d1x = x[i] - zc, d1y = y[i] - rc, d2x = x[j] - zc, d2y = y[j] - rc;
    const double ex = x[j] - x[i], ey = y[j] - y[i];
    const double cross = d1x * d2y - d1y * d2x;
    const double P = fabs(d1x) + fabs(d1y) + fabs(d2x) + fabs(d2y) + fabs(ex) + fabs(ey);
    ok = ok && (fabs(cross) > 1e-4 * P * P);
  }
  return ok;
}

__device__ __forceinline__ void gather4(const int* nie, int e, int (&nid)[4]) {
  const int4 q = __ldg(reinterpret_cast<const int4*>(nie) + e);
  nid[0] = q.x;
  nid[1] = q.y;
  nid[2] = q.z;
  nid[3] = q.w;
}

// ---------------------------------------------------------------------------
// Corner forces of the quad (force_sgh.cpp:407-808).  The shock-direction and
// curl terms feed only unused values (use_shock_dir = 0, phi_curl unused) and
// are not computed.  STRENGTH: tau = stress(1) - p I and the hypo model with the
// RZ velocity gradient (momentum.cpp:151-217); otherwise stress is zero.
template <bool STRENGTH>
__global__ void __launch_bounds__(kRzBlock) k_force_rz(const RzForceArgs a) {
  if (!a.ctrl->active) return;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.ne) return;
  const int ne = a.ne;
  int nid[4];
  gather4(a.nie, e, nid);
  double x[4], y[4], u[4], v[4];
#pragma unroll
  for (int l = 0; l < 4; ++l) {
    x[l] = __ldg(a.x + nid[l]);
    y[l] = __ldg(a.y + nid[l]);
    u[l] = __ldg(a.u + nid[l]);
    v[l] = __ldg(a.v + nid[l]);
  }
  double B[4][2], ca[4] = {0.0, 0.0, 0.0, 0.0};
  rz_bmatrix(x, y, B);
  const double area = rz_area(x, y);
  const double den = a.den[e], pres = a.pres[e], sspd = a.sspd[e], vol = a.vol[e], div = a.div[e];
  const bool hoop_zero = !STRENGTH && isfinite(pres) && rz_corner_areas_finite(x, y);
  if (!hoop_zero) rz_corner_areas(x, y, ca);
  const int mat = a.mat[e];
  const double* q = a.qtab + 4 * mat;
  const bool compress = div < 0;
  const double qa = compress ? q[0] : q[1];
  const double qb = compress ? q[2] : q[3];
  // Cauchy stress (:480-493): tau(i,j) = stress(i,j), tau(i,i) -= p
  double sc[9], t[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    sc[k] = STRENGTH ? a.stress_cur[(size_t)k * ne + e] : 0.0;
    t[k] = sc[k];
  }
  t[0] = t[0] - pres;
  t[4] = t[4] - pres;
  t[8] = t[8] - pres;
  // average velocity (:500-512); 0.25*v is exact, so fusing equals product-then-add
  double vs0 = 0.0, vs1 = 0.0;
#pragma unroll
  for (int l = 0; l < 4; ++l) {
    vs0 = fma(0.25, u[l], vs0);
    vs1 = fma(0.25, v[l], vs1);
  }
  // MARS impedances (:520-636); |inward normal| = |B|
  double mu[4];
  double s0 = 0.0, s1 = 0.0, s3 = 0.0;
  const double q1c = qa * sspd;
#pragma unroll
  for (int l = 0; l < 4; ++l) {
    const double d0 = u[l] - vs0, d1 = v[l] - vs1;
    const double mag_vel = mode_sqrt(d0 * d0 + d1 * d1);
    const double muc = den * (q1c + qb * mag_vel);
    const double mu_term = muc * mode_sqrt(B[l][0] * B[l][0] + B[l][1] * B[l][1]);
    s0 = s0 + mu_term * u[l];
    s1 = s1 + mu_term * v[l];
    s3 = s3 + mu_term;
    mu[l] = mu_term;
  }
  double vstar0 = 0.0, vstar1 = 0.0;
  if (s3 > a.fuzz) {
#if FIERRO_FMA
    const double rs = mode_rcp(s3);
    vstar0 = s0 * rs;
    vstar1 = s1 * rs;
#else
    const Divisor ds3 = divisor(s3);  // correctly rounded quotients, one reciprocal seed
    vstar0 = quot(s0, ds3);
    vstar1 = quot(s1, ds3);
#endif
  }
  // shock detector (:653-690): the minimum over neighbours of the monotone
  // r_face(div_nb) sits at the smallest (div + small > 0) or largest neighbour
  // divergence, as in the 3D kernel
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
    if (isfinite(D) && D != 0.0 && isfinite(dsel)) {
      const double r_face = mode_div(0.9 * (dsel + small), D);
      r_min = okey(r_face) < okey(1.0) ? r_face : 1.0;
    } else {
      for (int k = k0; k < k1; ++k) {
        const double r_face = mode_div(0.9 * (__ldg(a.div + __ldg(a.eie + k)) + small), D);
        r_min = fmin(r_face, r_min);
      }
    }
  }
  double phi = 1.0 - fmax(0.0, r_min);
  // Mach-number detector with the characteristic length sqrt(area) (:692-700)
  const double c_length = mode_sqrt(area);
  const double alpha = fmin(1.0, mode_div(20.0 * (c_length * fabs(div)), sspd + a.fuzz));
  phi = alpha * phi;
  // corner forces with the inward normals -B, then the hoop-stress terms (:718-755)
  const double vs[2] = {vstar0, vstar1};
#pragma unroll
  for (int l = 0; l < 4; ++l) {
    const double pm = phi * mu[l];
    const double a0 = -B[l][0], a1 = -B[l][1];
    const double vl[2] = {u[l], v[l]};
    double f[2];
#pragma unroll
    for (int d = 0; d < 2; ++d) f[d] = a0 * t[d] + a1 * t[3 + d] + pm * (vs[d] - vl[d]);
    const double r = y[l];
    if (r > 1e-14) {
      if (hoop_zero) {
        // the terms' exact value (+0.0 turns a -0.0 force into +0.0, as adding them does)
        f[0] = f[0] + 0.0;
        f[1] = f[1] + 0.0;
      } else {
        f[0] = f[0] + t[3] * ca[l] / r;
        f[1] = f[1] + (t[4] - t[8]) * ca[l] / r;
      }
    }
    a.force[(size_t)(l * 2 + 0) * ne + e] = f[0];
    a.force[(size_t)(l * 2 + 1) * ne + e] = f[1];
  }
  if (STRENGTH) {
    if (a.stype[mat] == 1) {
      // get_velgrad2D (momentum.cpp:151-217) with the outward normals
      double L[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) L[k] = 0.0;
      const double mean_radius = vol / area;
      const double elem_vel_r = 0.25 * (v[0] + v[1] + v[2] + v[3]);
      const double inverse_area = 1.0 / area;
      L[0] = (u[0] * B[0][0] + u[1] * B[1][0] + u[2] * B[2][0] + u[3] * B[3][0]) * inverse_area;
      L[1] = (u[0] * B[0][1] + u[1] * B[1][1] + u[2] * B[2][1] + u[3] * B[3][1]) * inverse_area;
      L[3] = (v[0] * B[0][0] + v[1] * B[1][0] + v[2] * B[2][0] + v[3] * B[3][0]) * inverse_area;
      L[4] = (v[0] * B[0][1] + v[1] * B[1][1] + v[2] * B[2][1] + v[3] * B[3][1]) * inverse_area;
      L[8] = elem_vel_r / mean_radius;
      double s0v[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) s0v[k] = a.stress0[(size_t)k * ne + e];
      user_strength_model(sc, s0v, L, a.statev + e, ne, mat, den, a.sie0[e], vol, a.ctrl->dt, a.rk_alpha);
#pragma unroll
      for (int k = 0; k < 9; ++k) a.stress_out[(size_t)k * ne + e] = sc[k];
    } else if (a.copy_stress) {
#pragma unroll
      for (int k = 0; k < 9; ++k) a.stress_out[(size_t)k * ne + e] = sc[k];
    }
  }
}

// ---------------------------------------------------------------------------
// Node update.  The velocity uses the areal mass the previous stage left; the
// mass of the new position replaces it at the end (the reference recomputes it
// after update_state2D, and nothing in between reads it).
__global__ void __launch_bounds__(kRzNodeBlock) k_node_rz(const RzNodeArgs a) {
  if (!a.ctrl->active) return;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= a.nn) return;
  const size_t ne = (size_t)a.ne;
  double f0 = 0.0, f1 = 0.0;
  const int c0 = a.cin_start[n], c1 = a.cin_start[n + 1];
  for (int c = c0; c < c1; ++c) {
    const int cid = __ldg(a.cin + c);
    const int e = cid >> 2, l = cid & 3;
    f0 = f0 + __ldg(a.force + (size_t)(l * 2 + 0) * ne + e);
    f1 = f1 + __ldg(a.force + (size_t)(l * 2 + 1) * ne + e);
  }
  const double adt = a.rk_alpha * a.ctrl->dt;
  const double m = a.node_mass[n];
  const double u0 = a.u0[n], v0 = a.v0[n];
#if FIERRO_FMA
  const double rm = mode_rcp(m);
  double u1 = u0 + adt * f0 * rm;
  double v1 = v0 + adt * f1 * rm;
#else
  const Divisor dm = divisor(m);  // correctly rounded quotients, one reciprocal seed
  double u1 = u0 + quot(adt * f0, dm);
  double v1 = v0 + quot(adt * f1, dm);
#endif
  const unsigned bc = a.bc_mask[n];
  if (bc & 1u) u1 = 0.0;
  if (bc & 2u) v1 = 0.0;
  const double hu = (u1 + u0) * 0.5, hv = (v1 + v0) * 0.5;
  const double r_in = a.yin[n];  // read before y1 is overwritten (yin == y1 after the first stage)
  a.u1[n] = u1;
  a.v1[n] = v1;
  a.hx[n] = hu;
  a.hy[n] = hv;
  a.rad[n] = r_in;
  const double x1 = a.x0[n] + adt * hu;
  const double y1 = a.y0[n] + adt * hv;
  a.x1[n] = x1;
  a.y1[n] = y1;
  double mn = 0.0;
  if (y1 > a.tiny) mn = a.node_ext[n] / y1;
  a.node_mass[n] = mn;
}

// Nodes on the axis (y < tiny) among the boundary nodes: the largest half-mass
// of their off-axis edge neighbours.  Off-axis masses are not written here.
__global__ void __launch_bounds__(kRzNodeBlock) k_axis_rz(const RzAxisArgs a) {
  if (!a.ctrl->active) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.naxis) return;
  const int n = a.nodes[i];
  if (!(a.y1[n] < a.tiny)) return;
  double m = a.node_mass[n];
  for (int k = a.nin_start[i]; k < a.nin_start[i + 1]; ++k) {
    const int nb = a.nin[k];
    if (a.y1[nb] > a.tiny) m = fmax(m, a.node_mass[nb] / 2.0);
  }
  a.node_mass[n] = m;
}

// ---------------------------------------------------------------------------
template <int KIND>
__global__ void __launch_bounds__(kRzBlock) k_elem_rz(const RzElemArgs a) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  Ctrl* ctrl = a.ctrl;
  if (KIND != 2 && !ctrl->active) return;
  long long dkey = 0x7FFFFFFFFFFFFFFFLL;
  if (e < a.ne) {
    const int ne = a.ne;
    int nid[4];
    gather4(a.nie, e, nid);
    double x[4], y[4], u[4], v[4];
#pragma unroll
    for (int l = 0; l < 4; ++l) {
      x[l] = __ldg(a.x + nid[l]);
      y[l] = __ldg(a.y + nid[l]);
      u[l] = __ldg(a.u + nid[l]);
      v[l] = __ldg(a.v + nid[l]);
    }
    double sie1 = 0.0;
    if (KIND != 2) {
      // energy (energy_sgh.cpp:16-52): power = sum_c F_c r_c (v1 + v0)/2 with the
      // node radius of the stage's input state
      double power = 0.0;
#pragma unroll
      for (int l = 0; l < 4; ++l) {
        const double r = __ldg(a.rad + nid[l]);
        power = power + a.force[(size_t)(l * 2 + 0) * ne + e] * r * __ldg(a.hx + nid[l]);
        power = power + a.force[(size_t)(l * 2 + 1) * ne + e] * r * __ldg(a.hy + nid[l]);
      }
      const double adt = a.rk_alpha * ctrl->dt;
      sie1 = a.sie0[e] - mode_div(adt, a.mass[e]) * power;
      a.sie1[e] = sie1;
    }
    const double vol = (KIND == 2) ? a.vol[e] : rz_vol(x, y);
    // divergence for the next stage (momentum.cpp:298-378)
    double B[4][2];
    rz_bmatrix(x, y, B);
    const double area = rz_area(x, y);
    const double inverse_area = mode_rcp(area);
    const double mean_radius = mode_div(vol, area);
    const double elem_vel_r = 0.25 * (v[0] + v[1] + v[2] + v[3]);
    double div = 0.0;
    div = div + (u[0] * B[0][0] + u[1] * B[1][0] + u[2] * B[2][0] + u[3] * B[3][0]) * inverse_area;
    div = div + ((v[0] * B[0][1] + v[1] * B[1][1] + v[2] * B[2][1] + v[3] * B[3][1]) * inverse_area +
                 mode_div(elem_vel_r, mean_radius));
    a.div[e] = div;
    double sspd;
    if (KIND != 2) {
      a.vol[e] = vol;
      // update_state2D (properties.cpp:140, eos.cpp:12-46)
      const double den = mode_div(a.mass[e], vol);
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
      // CFL step (time_integration.cpp:189-228): the six node-pair distances; the
      // minimum of the square roots is the square root of the minimum
      double d2 = 0.0;
      bool first = true;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = i + 1; j <= 3; ++j) {
          const double dx = x[i] - x[j], dy = y[i] - y[j];
          const double s = dx * dx + dy * dy;
          d2 = first ? s : fmin(s, d2);
          first = false;
        }
      const double dist_min = mode_sqrt(d2);
      const double dt_l = mode_div(a.dt_cfl * dist_min, sspd + a.fuzz);
      dkey = isnan(dt_l) ? 0x7FFFFFFFFFFFFFFFLL : okey(dt_l);
    }
  }
  if (KIND != 0) {
    const long long k = block_min_key(dkey);
    if (threadIdx.x == 0) a.cfl_part[blockIdx.x] = k;
  }
}

__global__ void __launch_bounds__(kRzNodeBlock) k_ext_rz(int nn, const double* node_mass, const double* y,
                                                        double* ext) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n < nn) ext[n] = node_mass[n] * y[n];
}

// Energy tallies (sgh_solve.cpp:73-101): IE = sum M e, KE = 1/2 sum m y |v|^2.
constexpr int kRzEnergyBlock = 256;
__global__ void __launch_bounds__(kRzEnergyBlock) k_energy_rz_part(const RzEnergyArgs a) {
  __shared__ double sh[2][kRzEnergyBlock];
  double ie = 0.0, ke = 0.0;
  const int stride = gridDim.x * blockDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.ne; i += stride) ie += a.mass[i] * a.sie[i];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nn; i += stride) {
    double k = 0;
    k += a.u[i] * a.u[i];
    k += a.v[i] * a.v[i];
    ke += a.node_mass[i] * a.y[i] * k;
  }
  sh[0][threadIdx.x] = ie;
  sh[1][threadIdx.x] = ke;
  __syncthreads();
  for (int s = kRzEnergyBlock / 2; s > 0; s >>= 1) {
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

__global__ void k_energy_rz_final(const RzEnergyArgs a, int nblocks) {
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

static void launch_force(const RzForceArgs& a, cudaStream_t s) {
  if (a.stress_out) k_force_rz<true><<<blocks_for(a.ne, kRzBlock), kRzBlock, 0, s>>>(a);
  else k_force_rz<false><<<blocks_for(a.ne, kRzBlock), kRzBlock, 0, s>>>(a);
}
static void launch_node(const RzNodeArgs& a, cudaStream_t s) {
  k_node_rz<<<blocks_for(a.nn, kRzNodeBlock), kRzNodeBlock, 0, s>>>(a);
}
static void launch_axis(const RzAxisArgs& a, cudaStream_t s) {
  k_axis_rz<<<blocks_for(a.naxis > 0 ? a.naxis : 1, kRzNodeBlock), kRzNodeBlock, 0, s>>>(a);
}
static void launch_elem(const RzElemArgs& a, int kind, cudaStream_t s) {
  const unsigned g = blocks_for(a.ne, kRzBlock);
  if (kind == 0) k_elem_rz<0><<<g, kRzBlock, 0, s>>>(a);
  else if (kind == 1) k_elem_rz<1><<<g, kRzBlock, 0, s>>>(a);
  else k_elem_rz<2><<<g, kRzBlock, 0, s>>>(a);
}
static void launch_ext(int nn, const double* node_mass, const double* y, double* ext, cudaStream_t s) {
  k_ext_rz<<<blocks_for(nn, kRzNodeBlock), kRzNodeBlock, 0, s>>>(nn, node_mass, y, ext);
}
static void launch_energy(const RzEnergyArgs& a, cudaStream_t s) {
  const int nb = 512;
  k_energy_rz_part<<<nb, kRzEnergyBlock, 0, s>>>(a);
  k_energy_rz_final<<<1, 32, 0, s>>>(a, nb);
}

}  // namespace FIERRO_RZ_IMPL

#if FIERRO_FMA
const RzKernelSet& rz_kernels_fma() {
  static const RzKernelSet k = {rz_fma_impl::launch_force, rz_fma_impl::launch_node, rz_fma_impl::launch_axis,
                                rz_fma_impl::launch_elem, rz_fma_impl::launch_ext, rz_fma_impl::launch_energy};
  return k;
}
#else
const RzKernelSet& rz_kernels_exact() {
  static const RzKernelSet k = {rz_exact_impl::launch_force, rz_exact_impl::launch_node,
                                rz_exact_impl::launch_axis, rz_exact_impl::launch_elem,
                                rz_exact_impl::launch_ext, rz_exact_impl::launch_energy};
  return k;
}
#endif

}  // namespace fierro
