/* CPU oracle for the 2D-RZ SGH cycle: a plain-C restatement of the axisymmetric
 * (num_dims == 2) branches of Fierro's Explicit-Lagrange-Kokkos/SGH_solver.
 *
 * TEST INFRASTRUCTURE ONLY, like oracle/sgh_oracle.c: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU baseline leg may load it, and only
 * as the checker.  The GB300 library never links or calls it.
 *
 * Each function restates the reference's operations with the same operands in
 * the same association order (compiled with -ffp-contract=off); the comments
 * cite the reference file:line restated.  Coordinates are (x axial, y radial);
 * quads are counter-clockwise (sgh_solve.cpp:513-519).  Layouts:
 *   node_coords, node_vel  [2][num_nodes][2]
 *   corner_force           [4*num_elems][2]   corner gid = elem*4 + node_lid
 *   elem_stress            [2][num_elems][3][3]
 *   nodes_in_elem          [num_elems][4]
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "sgh_oracle.h"

struct orc_rz {
  int64_t nn, ne;
  int64_t* nie;        /* [ne][4] */
  int64_t* cin_start;  /* corners_in_node CSR, ascending corner gid (mesh.h:180-245) */
  int64_t* cin;
  int64_t* eie_start;  /* elems_in_elem: every other element sharing a node (mesh.h:249-338) */
  int64_t* eie;
  int64_t* nin_start;  /* nodes_in_node: the two ends of every edge (mesh.h:654-796) */
  int64_t* nin;
  int64_t nbdy;        /* bdy_nodes: nodes on an edge owned by one element (mesh.h:592-645) */
  int64_t* bdy_nodes;
  int nsets;
  int64_t* bset_start; /* bdy_nodes_in_set CSR */
  int64_t* bset;
  int nmat, nsv;
  orc_material* mat;
  double* state_vars;
  orc_boundary* bc;
  double *coords, *vel, *node_mass, *node_ext_mass;
  double *den, *pres, *stress, *sspd, *sie, *vol, *div, *mass, *statev;
  int64_t* mat_id;
  double* corner_force;
  double time_value, dt, graphics_time;
  int64_t cycle;
  int stage;
  int stopped;
  int ext_valid; /* node_extensive_mass computed for the current run (sgh_solve.cpp:106-114) */
};

#define X1(s, n, d) ((s)->coords[(size_t)(s)->nn * 2 + (size_t)(n) * 2 + (d)])
#define X0(s, n, d) ((s)->coords[(size_t)(n) * 2 + (d)])
#define V1(s, n, d) ((s)->vel[(size_t)(s)->nn * 2 + (size_t)(n) * 2 + (d)])
#define V0(s, n, d) ((s)->vel[(size_t)(n) * 2 + (d)])

/* quad edges as patches (mesh.h:364-373) */
static const int RZ_EDGE[4][2] = {{0, 3}, {1, 2}, {0, 1}, {3, 2}};

static void* zalloc(size_t n) { return calloc(n ? n : 1, 1); }

/* The CFL distance's pow(d, 2.0) (time_integration.cpp:208-209): libm pow by
 * default, the IEEE square d*d with -DORC_CR_POW (as in sgh_oracle.c). */
static double rz_pow2(double d) {
#ifdef ORC_CR_POW
  return d * d;
#else
  return pow(d, 2.0);
#endif
}

/* ---- geometry (geometry.cpp:314-547) ------------------------------------- */

/* get_bmatrix2D, geometry.cpp:315-365: outward corner normals B[l][dim]. */
void orc_rz_bmatrix(const double x[4], const double y[4], double B[4][2]) {
  B[0][0] = -0.5 * (y[3] - y[1]);
  B[1][0] = -0.5 * (y[0] - y[2]);
  B[2][0] = -0.5 * (y[1] - y[3]);
  B[3][0] = -0.5 * (y[2] - y[0]);
  B[0][1] = -0.5 * (x[1] - x[3]);
  B[1][1] = -0.5 * (x[2] - x[0]);
  B[2][1] = -0.5 * (x[3] - x[1]);
  B[3][1] = -0.5 * (x[0] - x[2]);
}

/* get_vol_quad, geometry.cpp:369-434: volume per radian of the revolved quad. */
double orc_rz_vol_quad(const double x[4], const double y[4]) {
  return ((y[2] + y[3] + y[0]) * ((y[2] - y[3]) * (x[0] - x[3]) - (y[0] - y[3]) * (x[2] - x[3])) +
          (y[0] + y[1] + y[2]) * ((y[0] - y[1]) * (x[2] - x[1]) - (y[2] - y[1]) * (x[0] - x[1]))) /
         6.0;
}

/* get_area_quad, geometry.cpp:438-466 */
double orc_rz_area_quad(const double x[4], const double y[4]) {
  return 0.5 * ((x[0] - x[2]) * (y[1] - y[3]) + (x[3] - x[1]) * (y[0] - y[2]));
}

/* heron, geometry.cpp:470-500 */
static double heron(double x1, double y1, double x2, double y2, double x3, double y3) {
  double S = 0.0, a, b, c;
  a = sqrt((x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1));
  S += a;
  b = sqrt((x3 - x2) * (x3 - x2) + (y3 - y2) * (y3 - y2));
  S += b;
  c = sqrt((x3 - x1) * (x3 - x1) + (y3 - y1) * (y3 - y1));
  S += c;
  S *= 0.5;
  return sqrt(S * (S - a) * (S - b) * (S - c));
}

/* get_area_weights2D, geometry.cpp:503-547: corner areas of Barlow's partition. */
void orc_rz_corner_areas(const double x[4], const double y[4], double ca[4]) {
  double rc = 0.0, zc = 0.0;
  for (int l = 0; l < 4; ++l) {
    rc += 0.25 * y[l];
    zc += 0.25 * x[l];
  }
  double A12 = heron(x[0], y[0], zc, rc, x[1], y[1]);
  double A23 = heron(x[1], y[1], zc, rc, x[2], y[2]);
  double A34 = heron(x[2], y[2], zc, rc, x[3], y[3]);
  double A41 = heron(x[3], y[3], zc, rc, x[0], y[0]);
  ca[0] = (5. * A41 + 5. * A12 + A23 + A34) / 12.;
  ca[1] = (A41 + 5. * A12 + 5. * A23 + A34) / 12.;
  ca[2] = (A41 + A12 + 5. * A23 + 5. * A34) / 12.;
  ca[3] = (5. * A41 + A12 + A23 + 5. * A34) / 12.;
}

static void gather(const orc_rz* s, int64_t e, double x[4], double y[4]) {
  for (int l = 0; l < 4; ++l) {
    int64_t n = s->nie[e * 4 + l];
    x[l] = X1(s, n, 0);
    y[l] = X1(s, n, 1);
  }
}

/* ---- topology -------------------------------------------------------------- */

static int cmp_pair(const void* a, const void* b) {
  const int64_t* x = (const int64_t*)a;
  const int64_t* y = (const int64_t*)b;
  if (x[0] != y[0]) return (x[0] > y[0]) - (x[0] < y[0]);
  return (x[1] > y[1]) - (x[1] < y[1]);
}

static void build_topology(orc_rz* s) {
  const int64_t nn = s->nn, ne = s->ne;
  s->cin_start = (int64_t*)zalloc(sizeof(int64_t) * (size_t)(nn + 1));
  for (int64_t i = 0; i < ne * 4; ++i) s->cin_start[s->nie[i] + 1]++;
  for (int64_t n = 0; n < nn; ++n) s->cin_start[n + 1] += s->cin_start[n];
  s->cin = (int64_t*)zalloc(sizeof(int64_t) * (size_t)(4 * ne));
  int64_t* fill = (int64_t*)zalloc(sizeof(int64_t) * (size_t)nn);
  for (int64_t e = 0; e < ne; ++e)
    for (int l = 0; l < 4; ++l) {
      int64_t n = s->nie[e * 4 + l];
      s->cin[s->cin_start[n] + fill[n]++] = e * 4 + l;
    }
  free(fill);
  /* neighbours */
  s->eie_start = (int64_t*)zalloc(sizeof(int64_t) * (size_t)(ne + 1));
  int64_t* tmp = (int64_t*)zalloc(sizeof(int64_t) * (size_t)ne * 32);
  int64_t* cnt = (int64_t*)zalloc(sizeof(int64_t) * (size_t)ne);
  for (int64_t e = 0; e < ne; ++e) {
    int64_t* row = tmp + e * 32;
    int64_t k = 0;
    for (int l = 0; l < 4; ++l) {
      int64_t n = s->nie[e * 4 + l];
      for (int64_t c = s->cin_start[n]; c < s->cin_start[n + 1]; ++c) {
        int64_t nb = s->cin[c] / 4;
        if (nb == e) continue;
        int seen = 0;
        for (int64_t i = 0; i < k; ++i)
          if (row[i] == nb) { seen = 1; break; }
        if (!seen && k < 32) row[k++] = nb;
      }
    }
    cnt[e] = k;
  }
  for (int64_t e = 0; e < ne; ++e) s->eie_start[e + 1] = s->eie_start[e] + cnt[e];
  s->eie = (int64_t*)zalloc(sizeof(int64_t) * (size_t)s->eie_start[ne]);
  for (int64_t e = 0; e < ne; ++e)
    memcpy(s->eie + s->eie_start[e], tmp + e * 32, sizeof(int64_t) * (size_t)cnt[e]);
  free(tmp);
  free(cnt);
  /* edges: sorted (min, max, elem, edge) records; an edge seen once is a boundary patch */
  int64_t* rec = (int64_t*)zalloc(sizeof(int64_t) * (size_t)ne * 4 * 4);
  for (int64_t e = 0; e < ne; ++e)
    for (int p = 0; p < 4; ++p) {
      int64_t a = s->nie[e * 4 + RZ_EDGE[p][0]], b = s->nie[e * 4 + RZ_EDGE[p][1]];
      int64_t* r = rec + (e * 4 + p) * 4;
      r[0] = a < b ? a : b;
      r[1] = a < b ? b : a;
      r[2] = e;
      r[3] = p;
    }
  qsort(rec, (size_t)ne * 4, sizeof(int64_t) * 4, cmp_pair);
  int64_t* deg = (int64_t*)zalloc(sizeof(int64_t) * (size_t)nn);
  char* on_bdy = (char*)zalloc((size_t)nn);
  for (int64_t i = 0; i < ne * 4;) {
    int64_t j = i + 1;
    while (j < ne * 4 && rec[j * 4] == rec[i * 4] && rec[j * 4 + 1] == rec[i * 4 + 1]) ++j;
    deg[rec[i * 4]]++;
    deg[rec[i * 4 + 1]]++;
    if (j - i == 1) on_bdy[rec[i * 4]] = on_bdy[rec[i * 4 + 1]] = 1;
    i = j;
  }
  s->nin_start = (int64_t*)zalloc(sizeof(int64_t) * (size_t)(nn + 1));
  for (int64_t n = 0; n < nn; ++n) s->nin_start[n + 1] = s->nin_start[n] + deg[n];
  s->nin = (int64_t*)zalloc(sizeof(int64_t) * (size_t)s->nin_start[nn]);
  memset(deg, 0, sizeof(int64_t) * (size_t)nn);
  for (int64_t i = 0; i < ne * 4;) {
    int64_t j = i + 1;
    while (j < ne * 4 && rec[j * 4] == rec[i * 4] && rec[j * 4 + 1] == rec[i * 4 + 1]) ++j;
    int64_t a = rec[i * 4], b = rec[i * 4 + 1];
    s->nin[s->nin_start[a] + deg[a]++] = b;
    s->nin[s->nin_start[b] + deg[b]++] = a;
    i = j;
  }
  free(deg);
  free(rec);
  s->nbdy = 0;
  for (int64_t n = 0; n < nn; ++n) s->nbdy += on_bdy[n];
  s->bdy_nodes = (int64_t*)zalloc(sizeof(int64_t) * (size_t)s->nbdy);
  int64_t k = 0;
  for (int64_t n = 0; n < nn; ++n)
    if (on_bdy[n]) s->bdy_nodes[k++] = n;
  free(on_bdy);
}

orc_rz* orc_rz_create(int64_t num_nodes, int64_t num_elems, const int64_t* nodes_in_elem,
                      const double* coords) {
  if (num_nodes <= 0 || num_elems <= 0 || !nodes_in_elem || !coords) return NULL;
  for (int64_t i = 0; i < num_elems * 4; ++i)
    if (nodes_in_elem[i] < 0 || nodes_in_elem[i] >= num_nodes) return NULL;
  orc_rz* s = (orc_rz*)zalloc(sizeof(orc_rz));
  s->nn = num_nodes;
  s->ne = num_elems;
  size_t nn = (size_t)num_nodes, ne = (size_t)num_elems;
  s->nie = (int64_t*)zalloc(sizeof(int64_t) * ne * 4);
  memcpy(s->nie, nodes_in_elem, sizeof(int64_t) * ne * 4);
  s->coords = (double*)zalloc(sizeof(double) * 2 * nn * 2);
  s->vel = (double*)zalloc(sizeof(double) * 2 * nn * 2);
  s->node_mass = (double*)zalloc(sizeof(double) * nn);
  s->node_ext_mass = (double*)zalloc(sizeof(double) * nn);
  memcpy(s->coords, coords, sizeof(double) * nn * 2);
  memcpy(s->coords + nn * 2, coords, sizeof(double) * nn * 2);
  s->den = (double*)zalloc(sizeof(double) * ne);
  s->pres = (double*)zalloc(sizeof(double) * ne);
  s->stress = (double*)zalloc(sizeof(double) * 2 * ne * 9);
  s->sspd = (double*)zalloc(sizeof(double) * ne);
  s->sie = (double*)zalloc(sizeof(double) * 2 * ne);
  s->vol = (double*)zalloc(sizeof(double) * ne);
  s->div = (double*)zalloc(sizeof(double) * ne);
  s->mass = (double*)zalloc(sizeof(double) * ne);
  s->mat_id = (int64_t*)zalloc(sizeof(int64_t) * ne);
  s->corner_force = (double*)zalloc(sizeof(double) * ne * 8);
  build_topology(s);
  return s;
}

void orc_rz_destroy(orc_rz* s) {
  if (!s) return;
  free(s->nie); free(s->cin_start); free(s->cin); free(s->eie_start); free(s->eie);
  free(s->nin_start); free(s->nin); free(s->bdy_nodes); free(s->bset_start); free(s->bset);
  free(s->mat); free(s->state_vars); free(s->bc); free(s->coords); free(s->vel);
  free(s->node_mass); free(s->node_ext_mass); free(s->den); free(s->pres); free(s->stress);
  free(s->sspd); free(s->sie); free(s->vol); free(s->div); free(s->mass); free(s->statev);
  free(s->mat_id); free(s->corner_force);
  free(s);
}

/* Hyper models are refused: update_state2D (properties.cpp:146-160) calls the 3D
 * get_bmatrix into an 8-entry array, which writes past its end. */
int orc_rz_set_materials(orc_rz* s, int num_materials, const orc_material* m, int num_state_vars,
                         const double* state_vars) {
  if (num_materials <= 0 || num_state_vars < 2) return 1;
  for (int i = 0; i < num_materials; ++i) {
    if (m[i].eos_model != 0 || m[i].strength_type < 0 || m[i].strength_type > 1) return 1;
    if (m[i].strength_type != 0 && num_state_vars < 4) return 1;
  }
  free(s->mat); free(s->state_vars); free(s->statev);
  s->nmat = num_materials;
  s->nsv = num_state_vars;
  s->mat = (orc_material*)zalloc(sizeof(orc_material) * (size_t)num_materials);
  memcpy(s->mat, m, sizeof(orc_material) * (size_t)num_materials);
  s->state_vars = (double*)zalloc(sizeof(double) * (size_t)(num_materials * num_state_vars));
  memcpy(s->state_vars, state_vars, sizeof(double) * (size_t)(num_materials * num_state_vars));
  s->statev = (double*)zalloc(sizeof(double) * (size_t)s->ne * (size_t)num_state_vars);
  return 0;
}

/* Planes x and y, and cylinders sqrt(x^2 + y^2) = value; a z plane or a sphere
 * would read a third coordinate the 2D arrays do not have (boundary.cpp:38,
 * setup.cpp:528-560). */
int orc_rz_set_boundaries(orc_rz* s, int num_bcs, const orc_boundary* b) {
  if (num_bcs < 0) return 1;
  for (int i = 0; i < num_bcs; ++i) {
    if (b[i].hydro_bc < 0 || b[i].hydro_bc > 5) return 1; /* bdy_hydro_conds, mesh.h:910-918 */
    if (b[i].surface != 0 && b[i].surface != 1 && b[i].surface != 3) return 1;
    if (b[i].hydro_bc == 1 && b[i].surface == 3) return 1;
  }
  free(s->bc);
  s->nsets = num_bcs;
  s->bc = (orc_boundary*)zalloc(sizeof(orc_boundary) * (size_t)(num_bcs ? num_bcs : 1));
  if (num_bcs) memcpy(s->bc, b, sizeof(orc_boundary) * (size_t)num_bcs);
  return 0;
}

/* check_bdy (setup.cpp:487-571) for an edge, then tag_bdys / build_boundry_node_sets. */
static void build_bdy_sets(orc_rz* s) {
  const int64_t ne = s->ne, nn = s->nn;
  char* in = (char*)zalloc((size_t)nn * (size_t)(s->nsets ? s->nsets : 1));
  for (int64_t e = 0; e < ne; ++e)
    for (int p = 0; p < 4; ++p) {
      int64_t a = s->nie[e * 4 + RZ_EDGE[p][0]], b = s->nie[e * 4 + RZ_EDGE[p][1]];
      int shared = 0;
      for (int64_t c = s->cin_start[a]; c < s->cin_start[a + 1] && !shared; ++c) {
        int64_t o = s->cin[c] / 4;
        if (o == e) continue;
        for (int l = 0; l < 4; ++l)
          if (s->nie[o * 4 + l] == b) shared = 1;
      }
      if (shared) continue;
      for (int k = 0; k < s->nsets; ++k) {
        int on = 0;
        const int64_t pn[2] = {a, b};
        for (int q = 0; q < 2; ++q) {
          double c0 = X1(s, pn[q], 0), c1 = X1(s, pn[q], 1);
          int tag = s->bc[k].surface;
          double val = s->bc[k].value;
          if (tag == 0) { if (fabs(c0 - val) <= 1.0e-7) on += 1; }
          else if (tag == 1) { if (fabs(c1 - val) <= 1.0e-7) on += 1; }
          else if (tag == 3) { double R = sqrt(c0 * c0 + c1 * c1); if (fabs(R - val) <= 1.0e-7) on += 1; }
        }
        if (on == 2) in[(size_t)k * (size_t)nn + (size_t)a] = in[(size_t)k * (size_t)nn + (size_t)b] = 1;
      }
    }
  free(s->bset_start); free(s->bset);
  s->bset_start = (int64_t*)zalloc(sizeof(int64_t) * (size_t)(s->nsets + 1));
  int64_t total = 0;
  for (size_t i = 0; i < (size_t)nn * (size_t)s->nsets; ++i) total += in[i];
  s->bset = (int64_t*)zalloc(sizeof(int64_t) * (size_t)total);
  int64_t k = 0;
  for (int b = 0; b < s->nsets; ++b) {
    for (int64_t n = 0; n < nn; ++n)
      if (in[(size_t)b * (size_t)nn + (size_t)n]) s->bset[k++] = n;
    s->bset_start[b + 1] = k;
  }
  free(in);
}

/* geometry.cpp:238-251 get_vol, 2D branch */
static void get_vol(orc_rz* s) {
  for (int64_t e = 0; e < s->ne; ++e) {
    double x[4], y[4];
    gather(s, e, x, y);
    s->vol[e] = orc_rz_vol_quad(x, y);
  }
}

/* eos.cpp:12-46 ideal_gas */
static void ideal_gas(orc_rz* s, int64_t e, double den, double sie) {
  double gamma = s->statev[e * s->nsv + 0];
  double csmin = s->statev[e * s->nsv + 1];
  s->pres[e] = (gamma - 1.0) * sie * den;
  s->sspd[e] = sqrt(gamma * (gamma - 1.0) * sie);
  if (s->sspd[e] < csmin) s->sspd[e] = csmin;
}

/* boundary.cpp:10-55 boundary_velocity with num_dims = 2 */
static void boundary_velocity(orc_rz* s) {
  for (int b = 0; b < s->nsets; ++b)
    for (int64_t k = s->bset_start[b]; k < s->bset_start[b + 1]; ++k) {
      int64_t n = s->bset[k];
      if (s->bc[b].hydro_bc == 1) V1(s, n, s->bc[b].surface) = 0.0;
      else if (s->bc[b].hydro_bc == 0)
        for (int d = 0; d < 2; ++d) V1(s, n, d) = 0.0;
    }
}

/* setup.cpp:10-424 with num_dims = 2 (get_vol first, driver.cpp:239). */
int orc_rz_setup(orc_rz* s, int num_fills, const orc_fill* fills) {
  if (!s->mat || (s->nsets > 0 && !s->bc)) return 1;
  for (int f = 0; f < num_fills; ++f) {
    if (fills[f].mat_id < 0 || fills[f].mat_id >= s->nmat) return 1;
    /* the spherical fill reads node_coords(rk, node, 2) past a 2D node's entries */
    if (fills[f].velocity == 2) return 1;
  }
  get_vol(s);
  build_bdy_sets(s);
  const int64_t ne = s->ne;
  const double PI = 3.141592653589793;
  for (int f = 0; f < num_fills; ++f) {
    const orc_fill* F = &fills[f];
    for (int64_t e = 0; e < ne; ++e) {
      double ec[3] = {0.0, 0.0, 0.0};
      for (int l = 0; l < 4; ++l) {
        int64_t n = s->nie[e * 4 + l];
        ec[0] += X1(s, n, 0);
        ec[1] += X1(s, n, 1);
        ec[2] = 0.0;
      }
      ec[0] = ec[0] / 4;
      ec[1] = ec[1] / 4;
      ec[2] = ec[2] / 4;
      double radius = sqrt(ec[0] * ec[0] + ec[1] * ec[1] + ec[2] * ec[2]);
      double radius_cyl = sqrt(ec[0] * ec[0] + ec[1] * ec[1]);
      int fill_this = 0;
      switch (F->volume) {
        case 0: fill_this = 1; break;
        case 1:
          if (ec[0] >= F->x1 && ec[0] <= F->x2 && ec[1] >= F->y1 && ec[1] <= F->y2 && ec[2] >= F->z1 &&
              ec[2] <= F->z2)
            fill_this = 1;
          break;
        case 2: if (radius_cyl >= F->radius1 && radius_cyl <= F->radius2) fill_this = 1; break;
        case 3: if (radius >= F->radius1 && radius <= F->radius2) fill_this = 1; break;
        default: break;
      }
      if (!fill_this) continue;
      s->den[e] = F->den;
      s->mass[e] = s->den[e] * s->vol[e];
      s->sie[ne + e] = F->sie;
      s->mat_id[e] = F->mat_id;
      for (int v = 0; v < s->nsv; ++v) s->statev[e * s->nsv + v] = s->state_vars[F->mat_id * s->nsv + v];
      for (int k = 0; k < 9; ++k) s->stress[(size_t)ne * 9 + (size_t)e * 9 + (size_t)k] = 0.0;
      ideal_gas(s, e, s->den[e], s->sie[ne + e]);
      for (int l = 0; l < 4; ++l) {
        int64_t n = s->nie[e * 4 + l];
        if (F->velocity == 0) {
          V1(s, n, 0) = F->u;
          V1(s, n, 1) = F->v;
        } else if (F->velocity == 1) {
          double dir[2] = {0.0, 0.0};
          double radius_val = 0.0;
          for (int d = 0; d < 2; ++d) {
            dir[d] = X1(s, n, d);
            radius_val += X1(s, n, d) * X1(s, n, d);
          }
          radius_val = sqrt(radius_val);
          for (int d = 0; d < 2; ++d) {
            if (radius_val > 1.0e-14) dir[d] /= (radius_val);
            else dir[d] = 0.0;
          }
          V1(s, n, 0) = F->speed * dir[0];
          V1(s, n, 1) = F->speed * dir[1];
        } else if (F->velocity == 5) {
          V1(s, n, 0) = sin(PI * X1(s, n, 0)) * cos(PI * X1(s, n, 1));
          V1(s, n, 1) = -1.0 * cos(PI * X1(s, n, 0)) * sin(PI * X1(s, n, 1));
        }
      }
      if (F->velocity == 5) {
        s->pres[e] = 0.25 * (cos(2.0 * PI * ec[0]) + cos(2.0 * PI * ec[1])) + 1.0;
        double gamma = s->statev[e * s->nsv + 4];
        s->sie[ne + e] = s->pres[e] / (F->den * (gamma - 1.0));
      }
    }
  }
  boundary_velocity(s);
  /* setup.cpp:365-420: corner masses (areal) and node mass summed in corner order */
  double* cmass = (double*)zalloc(sizeof(double) * (size_t)ne * 4);
  for (int64_t e = 0; e < ne; ++e) {
    double x[4], y[4], ca[4];
    gather(s, e, x, y);
    orc_rz_corner_areas(x, y, ca);
    for (int l = 0; l < 4; ++l) cmass[e * 4 + l] = ca[l] * s->den[e];
  }
  for (int64_t n = 0; n < s->nn; ++n) {
    double m = 0.0;
    for (int64_t c = s->cin_start[n]; c < s->cin_start[n + 1]; ++c) m += cmass[s->cin[c]];
    s->node_mass[n] = m;
  }
  free(cmass);
  return 0;
}

void orc_rz_init_time(orc_rz* s, const orc_params* p) {
  s->time_value = 0.0;
  s->dt = p->dt_start;
  s->graphics_time = p->graphics_dt_ival;
  s->cycle = 0;
  s->stage = 0;
  s->stopped = 0;
  s->ext_valid = 0;
}

/* time_integration.cpp:161-246 get_timestep2D */
static void get_timestep(orc_rz* s, const orc_params* p) {
  s->dt = s->dt * 1.1;
  double min_dt_calc = 1.7976931348623157e308;
  for (int64_t e = 0; e < s->ne; ++e) {
    double c[4][2], dist[6];
    for (int l = 0; l < 4; ++l)
      for (int d = 0; d < 2; ++d) c[l][d] = X1(s, s->nie[e * 4 + l], d);
    int count = 0;
    for (int i = 0; i < 3; ++i)
      for (int j = i + 1; j <= 3; ++j) {
        dist[count] = fabs(sqrt(rz_pow2(c[i][0] - c[j][0]) + rz_pow2(c[i][1] - c[j][1])));
        count++;
      }
    double dist_min = dist[0];
    for (int i = 0; i < 6; ++i) dist_min = fmin(dist[i], dist_min);
    double dt_l = p->dt_cfl * dist_min / (s->sspd[e] + p->fuzz);
    dt_l = fmin(dt_l, p->dt_max);
    dt_l = fmax(dt_l, p->dt_min);
    if (dt_l < min_dt_calc) min_dt_calc = dt_l;
  }
  if (min_dt_calc < s->dt) s->dt = min_dt_calc;
  s->dt = fmin(s->dt, (s->graphics_time - s->time_value) + p->fuzz);
  s->dt = fmin(s->dt, p->time_final - s->time_value);
}

/* time_integration.cpp:9-44 rk_init */
static void rk_init(orc_rz* s) {
  const size_t nn = (size_t)s->nn, ne = (size_t)s->ne;
  memcpy(s->stress, s->stress + ne * 9, sizeof(double) * ne * 9);
  memcpy(s->sie, s->sie + ne, sizeof(double) * ne);
  memcpy(s->coords, s->coords + nn * 2, sizeof(double) * nn * 2);
  memcpy(s->vel, s->vel + nn * 2, sizeof(double) * nn * 2);
}

/* momentum.cpp:298-378 get_divergence2D */
static void get_divergence(orc_rz* s) {
  for (int64_t e = 0; e < s->ne; ++e) {
    double x[4], y[4], B[4][2], u[4], v[4];
    gather(s, e, x, y);
    orc_rz_bmatrix(x, y, B);
    double elem_area = orc_rz_area_quad(x, y);
    for (int l = 0; l < 4; ++l) {
      int64_t n = s->nie[e * 4 + l];
      u[l] = V1(s, n, 0);
      v[l] = V1(s, n, 1);
    }
    double inverse_area = 1.0 / elem_area;
    double mean_radius = s->vol[e] / elem_area;
    double elem_vel_r = 0.25 * (v[0] + v[1] + v[2] + v[3]);
    double d = 0.0;
    d += (u[0] * B[0][0] + u[1] * B[1][0] + u[2] * B[2][0] + u[3] * B[3][0]) * inverse_area;
    d += (v[0] * B[0][1] + v[1] * B[1][1] + v[2] * B[2][1] + v[3] * B[3][1]) * inverse_area +
         elem_vel_r / mean_radius;
    s->div[e] = d;
  }
}

/* The test strength model of oracle/ref/ref_user_mat.cpp (G = statev(3)). */
static void strength_model(orc_rz* s, int64_t e, double L[3][3], double dt, double rk_alpha) {
  const size_t ne = (size_t)s->ne;
  const double G = s->statev[(size_t)e * (size_t)s->nsv + 3];
  double D[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) D[i][j] = 0.5 * (L[i][j] + L[j][i]);
  const double tr = D[0][0] + D[1][1] + D[2][2];
  for (int i = 0; i < 3; ++i) D[i][i] -= tr / 3.0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      s->stress[ne * 9 + (size_t)e * 9 + (size_t)(i * 3 + j)] =
          s->stress[(size_t)e * 9 + (size_t)(i * 3 + j)] + rk_alpha * dt * 2.0 * G * D[i][j];
}

/* force_sgh.cpp:407-808 get_force_sgh2D.  The shock-direction and curl terms
 * feed only unused values and are omitted. */
static void get_force(orc_rz* s, const orc_params* p, double rk_alpha) {
  const double fuzz = p->fuzz, small = p->small;
  const size_t ne = (size_t)s->ne;
  for (int64_t e = 0; e < s->ne; ++e) {
    double x[4], y[4], an[4][2], Bout[4][2], tau[3][3], muc[4], sum[4], vel_star[2], ca[4];
    gather(s, e, x, y);
    orc_rz_bmatrix(x, y, an);
    memcpy(Bout, an, sizeof(Bout));
    double elem_area = orc_rz_area_quad(x, y);
    orc_rz_corner_areas(x, y, ca);
    for (int l = 0; l < 4; ++l)
      for (int d = 0; d < 2; ++d) an[l][d] = (-1.0) * an[l][d];
    double div = s->div[e];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) tau[i][j] = s->stress[ne * 9 + (size_t)e * 9 + (size_t)(i * 3 + j)];
    for (int i = 0; i < 3; ++i) tau[i][i] -= s->pres[e];
    vel_star[0] = vel_star[1] = 0.0;
    for (int l = 0; l < 4; ++l) {
      int64_t n = s->nie[e * 4 + l];
      vel_star[0] += 0.25 * V1(s, n, 0);
      vel_star[1] += 0.25 * V1(s, n, 1);
    }
    for (int i = 0; i < 4; ++i) sum[i] = 0.0;
    const orc_material* M = &s->mat[s->mat_id[e]];
    for (int l = 0; l < 4; ++l) {
      int64_t n = s->nie[e * 4 + l];
      double v0 = V1(s, n, 0), v1 = V1(s, n, 1);
      double mag_vel = sqrt((v0 - vel_star[0]) * (v0 - vel_star[0]) + (v1 - vel_star[1]) * (v1 - vel_star[1]));
      if (div < 0) muc[l] = s->den[e] * (M->q1 * s->sspd[e] + M->q2 * mag_vel);
      else muc[l] = s->den[e] * (M->q1ex * s->sspd[e] + M->q2ex * mag_vel);
      double mu_term = muc[l] * sqrt(an[l][0] * an[l][0] + an[l][1] * an[l][1]);
      sum[0] += mu_term * v0;
      sum[1] += mu_term * v1;
      sum[3] += mu_term;
      muc[l] = mu_term;
    }
    if (sum[3] > fuzz) {
      for (int i = 0; i < 2; ++i) vel_star[i] = sum[i] / sum[3];
    } else {
      for (int i = 0; i < 2; ++i) vel_star[i] = 0.0;
    }
    double r_min = 1.0, r_coef = 0.9, n_coef = 1.0;
    for (int64_t k = s->eie_start[e]; k < s->eie_start[e + 1]; ++k) {
      double div_neighbor = s->div[s->eie[k]];
      double r_face = r_coef * (div_neighbor + small) / (div + small);
      r_min = fmin(r_face, r_min);
    }
    double phi = 1.0 - fmax(0.0, r_min);
    phi = pow(phi, n_coef);
    double omega = 20.0;
    double c_length = sqrt(elem_area);
    double alpha = fmin(1.0, omega * (c_length * fabs(div)) / (s->sspd[e] + fuzz));
    phi = alpha * phi;
    for (int l = 0; l < 4; ++l) {
      int64_t n = s->nie[e * 4 + l];
      double* F = &s->corner_force[((size_t)e * 4 + (size_t)l) * 2];
      for (int d = 0; d < 2; ++d)
        F[d] = an[l][0] * tau[0][d] + an[l][1] * tau[1][d] + phi * muc[l] * (vel_star[d] - V1(s, n, d));
      double node_radius = X1(s, n, 1);
      if (node_radius > 1e-14) {
        F[0] += tau[1][0] * ca[l] / node_radius;
        F[1] += (tau[1][1] - tau[2][2]) * ca[l] / node_radius;
      }
    }
    if (M->strength_type == 1) {
      /* momentum.cpp:151-217 get_velgrad2D */
      double u[4], v[4], L[3][3];
      for (int l = 0; l < 4; ++l) {
        int64_t n = s->nie[e * 4 + l];
        u[l] = V1(s, n, 0);
        v[l] = V1(s, n, 1);
      }
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) L[i][j] = 0.0;
      double mean_radius = s->vol[e] / elem_area;
      double elem_vel_r = 0.25 * (v[0] + v[1] + v[2] + v[3]);
      double inverse_area = 1.0 / elem_area;
      L[0][0] = (u[0] * Bout[0][0] + u[1] * Bout[1][0] + u[2] * Bout[2][0] + u[3] * Bout[3][0]) * inverse_area;
      L[0][1] = (u[0] * Bout[0][1] + u[1] * Bout[1][1] + u[2] * Bout[2][1] + u[3] * Bout[3][1]) * inverse_area;
      L[1][0] = (v[0] * Bout[0][0] + v[1] * Bout[1][0] + v[2] * Bout[2][0] + v[3] * Bout[3][0]) * inverse_area;
      L[1][1] = (v[0] * Bout[0][1] + v[1] * Bout[1][1] + v[2] * Bout[2][1] + v[3] * Bout[3][1]) * inverse_area;
      L[2][2] = elem_vel_r / mean_radius;
      strength_model(s, e, L, s->dt, rk_alpha);
    }
  }
}

/* momentum.cpp:11-53 update_velocity_sgh, num_dims = 2 */
static void update_velocity(orc_rz* s, double rk_alpha, double dt) {
  for (int64_t n = 0; n < s->nn; ++n) {
    double F[2] = {0.0, 0.0};
    for (int64_t c = s->cin_start[n]; c < s->cin_start[n + 1]; ++c)
      for (int d = 0; d < 2; ++d) F[d] += s->corner_force[(size_t)s->cin[c] * 2 + (size_t)d];
    for (int d = 0; d < 2; ++d) V1(s, n, d) = V0(s, n, d) + rk_alpha * dt * F[d] / s->node_mass[n];
  }
}

/* energy_sgh.cpp:6-55 update_energy_sgh: node_radius = node_coords(1, node, 1) */
static void update_energy(orc_rz* s, double rk_alpha, double dt) {
  const size_t ne = (size_t)s->ne;
  for (int64_t e = 0; e < s->ne; ++e) {
    double elem_power = 0.0;
    for (int l = 0; l < 4; ++l) {
      int64_t n = s->nie[e * 4 + l];
      double node_radius = X1(s, n, 1);
      for (int d = 0; d < 2; ++d) {
        double half_vel = (V1(s, n, d) + V0(s, n, d)) * 0.5;
        elem_power += s->corner_force[((size_t)e * 4 + (size_t)l) * 2 + (size_t)d] * node_radius * half_vel;
      }
    }
    s->sie[ne + (size_t)e] = s->sie[e] - rk_alpha * dt / s->mass[e] * elem_power;
  }
}

/* geometry.cpp:9-26 update_position_sgh, num_dims = 2 */
static void update_position(orc_rz* s, double rk_alpha, double dt) {
  for (int64_t n = 0; n < s->nn; ++n)
    for (int d = 0; d < 2; ++d) {
      double half_vel = (V1(s, n, d) + V0(s, n, d)) * 0.5;
      X1(s, n, d) = X0(s, n, d) + rk_alpha * dt * half_vel;
    }
}

/* properties.cpp:118-219 update_state2D (no hyper models) */
static void update_state(orc_rz* s) {
  const size_t ne = (size_t)s->ne;
  for (int64_t e = 0; e < s->ne; ++e) {
    s->den[e] = s->mass[e] / s->vol[e];
    ideal_gas(s, e, s->den[e], s->sie[ne + (size_t)e]);
  }
}

/* sgh_solve.cpp:494-581: areal node mass from the extensive mass, then nodes on
 * the axis take the largest half-mass of their off-axis edge neighbours. */
static void update_node_mass(orc_rz* s, double tiny) {
  for (int64_t n = 0; n < s->nn; ++n) {
    s->node_mass[n] = 0.0;
    if (X1(s, n, 1) > tiny) s->node_mass[n] = s->node_ext_mass[n] / X1(s, n, 1);
  }
  for (int64_t k = 0; k < s->nbdy; ++k) {
    int64_t n = s->bdy_nodes[k];
    if (X1(s, n, 1) < tiny)
      for (int64_t c = s->nin_start[n]; c < s->nin_start[n + 1]; ++c) {
        int64_t m = s->nin[c];
        if (X1(s, m, 1) > tiny) s->node_mass[n] = fmax(s->node_mass[n], s->node_mass[m] / 2.0);
      }
  }
}

static void rk_stage(orc_rz* s, const orc_params* p, int stage) {
  double rk_alpha = 1.0 / ((double)p->rk_num_stages - (double)stage);
  get_divergence(s);
  get_force(s, p, rk_alpha);
  update_velocity(s, rk_alpha, s->dt);
  boundary_velocity(s);
  update_energy(s, rk_alpha, s->dt);
  update_position(s, rk_alpha, s->dt);
  get_vol(s);
  update_state(s);
  update_node_mass(s, p->tiny);
}

static void end_cycle(orc_rz* s, const orc_params* p) {
  s->time_value += s->dt;
  int write = 0;
  if ((s->cycle + 1) % p->graphics_cyc_ival == 0 && s->cycle > 0) write = 1;
  else if (s->time_value >= p->time_final) write = 1;
  else if (s->time_value >= s->graphics_time) write = 1;
  if (write) s->graphics_time = s->time_value + p->graphics_dt_ival;
  if (s->time_value >= p->time_final) s->stopped = 1;
  s->cycle++;
}

int64_t orc_rz_run_stages(orc_rz* s, const orc_params* p, int64_t nstages) {
  if (!s->ext_valid) {
    /* sgh_solve.cpp:106-114: extensive node mass at the start of the run */
    for (int64_t n = 0; n < s->nn; ++n) s->node_ext_mass[n] = s->node_mass[n] * X1(s, n, 1);
    s->ext_valid = 1;
  }
  int64_t done = 0;
  while (done < nstages && !s->stopped) {
    if (s->stage == 0) {
      get_timestep(s, p);
      rk_init(s);
    }
    rk_stage(s, p, s->stage);
    s->stage++;
    done++;
    if (s->stage == (int)p->rk_num_stages) {
      s->stage = 0;
      end_cycle(s, p);
    }
  }
  return done;
}

int64_t orc_rz_run_cycles(orc_rz* s, const orc_params* p, int64_t ncycles) {
  int64_t c0 = s->cycle;
  for (int64_t c = 0; c < ncycles && !s->stopped; ++c) orc_rz_run_stages(s, p, p->rk_num_stages - s->stage);
  return s->cycle - c0;
}

/* sgh_solve.cpp:73-101: IE = sum M e, KE = 1/2 sum m y |v|^2 */
void orc_rz_energy(const orc_rz* s, double* ie, double* ke) {
  double IE = 0.0, KE = 0.0;
  for (int64_t e = 0; e < s->ne; ++e) IE += s->mass[e] * s->sie[(size_t)s->ne + (size_t)e];
  for (int64_t n = 0; n < s->nn; ++n) {
    double k = 0;
    for (int d = 0; d < 2; ++d) k += V1(s, n, d) * V1(s, n, d);
    KE += s->node_mass[n] * X1(s, n, 1) * k;
  }
  *ie = IE;
  *ke = 0.5 * KE;
}

void orc_rz_time(const orc_rz* s, double* time_value, double* dt, double* graphics_time, int64_t* cycle) {
  *time_value = s->time_value;
  *dt = s->dt;
  *graphics_time = s->graphics_time;
  *cycle = s->cycle;
}

static int64_t array_info(const orc_rz* s, int which, void** ptr, size_t* esize) {
  const int64_t nn = s->nn, ne = s->ne;
  *esize = sizeof(double);
  switch (which) {
    case ORC_NODE_COORDS: *ptr = s->coords; return 2 * nn * 2;
    case ORC_NODE_VEL: *ptr = s->vel; return 2 * nn * 2;
    case ORC_NODE_MASS: *ptr = s->node_mass; return nn;
    case ORC_ELEM_DEN: *ptr = s->den; return ne;
    case ORC_ELEM_PRES: *ptr = s->pres; return ne;
    case ORC_ELEM_STRESS: *ptr = s->stress; return 2 * ne * 9;
    case ORC_ELEM_SSPD: *ptr = s->sspd; return ne;
    case ORC_ELEM_SIE: *ptr = s->sie; return 2 * ne;
    case ORC_ELEM_VOL: *ptr = s->vol; return ne;
    case ORC_ELEM_DIV: *ptr = s->div; return ne;
    case ORC_ELEM_MASS: *ptr = s->mass; return ne;
    case ORC_ELEM_MAT_ID: *ptr = s->mat_id; *esize = sizeof(int64_t); return ne;
    case ORC_ELEM_STATEV: *ptr = s->statev; return ne * s->nsv;
    case ORC_CORNER_FORCE: *ptr = s->corner_force; return ne * 8;
    default: *ptr = NULL; return -1;
  }
}

int64_t orc_rz_get(const orc_rz* s, int which, void* out) {
  void* p;
  size_t es;
  int64_t n = array_info(s, which, &p, &es);
  if (n < 0 || !p) return -1;
  if (out) memcpy(out, p, (size_t)n * es);
  return n;
}

int64_t orc_rz_set(orc_rz* s, int which, const void* in) {
  void* p;
  size_t es;
  int64_t n = array_info(s, which, &p, &es);
  if (n < 0 || !p || !in) return -1;
  memcpy(p, in, (size_t)n * es);
  if (which == ORC_NODE_MASS || which == ORC_NODE_COORDS) s->ext_valid = 0;
  return n;
}
