/* CPU oracle for the SGH cycle -- plain-C restatement of Fierro's
 * Explicit-Lagrange-Kokkos/SGH_solver (3D hex, ideal gas, strength "none").
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GB300 library, never part of it.
 * Build with -ffp-contract=off so every double matches the reference's
 * uncontracted evaluation.  Parity of this file against the reference itself
 * (compiled from its own sources by oracle/build_ref.py) is pinned by
 * tests/test_oracle_ref.py and the fixtures in tests/golden/.
 */
#include "sgh_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------- */
/* Hex corner-normal cofactor tables (geometry.cpp:66-232, 298-306).
 * Corner p's outward area normal, component c, is
 *     B(p,c) = ( sum_t  O[j_t] * comb_t ) / 12
 * summed left to right over t = 0..5, where (O, I) = (y, z), (z, x), (x, y) for
 * c = 0, 1, 2 and comb_t = signed I-values summed left to right.  Terms are
 * encoded as +-(node+1), 0 = unused.  The volume (geometry.cpp:298-306) sums
 * x[i] * (sum_j y[j] * comb_ij) over i in HEX_V_I order with the j order of
 * HEX_V_J; its comb_ij are the B-matrix combos of (i, j). */
static const int HEX_B_J[8][6] = {
    {1, 2, 3, 4, 5, 7}, {0, 2, 3, 4, 5, 6}, {0, 1, 3, 5, 6, 7}, {0, 1, 2, 4, 6, 7},
    {0, 1, 3, 5, 6, 7}, {0, 1, 2, 4, 6, 7}, {1, 2, 3, 4, 5, 7}, {0, 2, 3, 4, 5, 6},
};
static const signed char HEX_B_TERMS[8][6][4] = {
    {{-3, -4, 5, 6}, {2, -4, 0, 0}, {2, 3, -5, -8}, {-2, 4, -6, 8}, {-2, 5, 0, 0}, {4, -5, 0, 0}},
    {{3, 4, -5, -6}, {-1, -4, 6, 7}, {-1, 3, 0, 0}, {1, -6, 0, 0}, {1, -3, 5, -7}, {-3, 6, 0, 0}},
    {{-2, 4, 0, 0}, {1, 4, -6, -7}, {-1, -2, 7, 8}, {2, -7, 0, 0}, {2, -4, 6, -8}, {-4, 7, 0, 0}},
    {{-2, -3, 5, 8}, {1, -3, 0, 0}, {1, 2, -7, -8}, {-1, 8, 0, 0}, {3, -8, 0, 0}, {-1, 3, -5, 7}},
    {{2, -4, 6, -8}, {-1, 6, 0, 0}, {1, -8, 0, 0}, {-1, -2, 7, 8}, {-6, 8, 0, 0}, {1, 4, -6, -7}},
    {{2, -5, 0, 0}, {-1, 3, -5, 7}, {-2, 7, 0, 0}, {1, 2, -7, -8}, {-2, -3, 5, 8}, {5, -7, 0, 0}},
    {{3, -6, 0, 0}, {-2, 4, -6, 8}, {-3, 8, 0, 0}, {6, -8, 0, 0}, {2, 3, -5, -8}, {-3, -4, 5, 6}},
    {{-4, 5, 0, 0}, {4, -7, 0, 0}, {1, -3, 5, -7}, {-1, -4, 6, 7}, {-5, 7, 0, 0}, {3, 4, -5, -6}},
};
static const int HEX_V_I[8] = {1, 7, 3, 5, 6, 0, 2, 4};
static const int HEX_V_J[8][6] = {
    {3, 4, 0, 6, 5, 2}, {0, 6, 2, 3, 5, 4}, {1, 7, 6, 2, 4, 0}, {0, 7, 2, 1, 4, 6},
    {1, 7, 5, 4, 3, 2}, {2, 7, 5, 1, 3, 4}, {0, 5, 1, 7, 6, 3}, {1, 7, 3, 0, 6, 5},
};
/* Patch (face) node lids, mesh.h:352-357. */
static const int HEX_PATCH[6][4] = {
    {0, 4, 7, 3}, {1, 2, 6, 5}, {0, 1, 5, 4}, {2, 3, 7, 6}, {0, 3, 2, 1}, {4, 5, 6, 7},
};

static double hex_comb(const signed char* t, const double* I) {
  double s = (t[0] > 0) ? I[t[0] - 1] : -I[-t[0] - 1];
  for (int k = 1; k < 4 && t[k] != 0; ++k) {
    if (t[k] > 0) s = s + I[t[k] - 1];
    else s = s - I[-t[k] - 1];
  }
  return s;
}

/* geometry.cpp:40-234 get_bmatrix: OUTWARD corner area normals. */
void orc_bmatrix(const double x[8], const double y[8], const double z[8], double B[8][3]) {
  const double twelth = 1. / 12.;
  const double* O[3] = {y, z, x};
  const double* I[3] = {z, x, y};
  for (int c = 0; c < 3; ++c) {
    for (int p = 0; p < 8; ++p) {
      double acc = O[c][HEX_B_J[p][0]] * hex_comb(HEX_B_TERMS[p][0], I[c]);
      for (int t = 1; t < 6; ++t) acc = acc + O[c][HEX_B_J[p][t]] * hex_comb(HEX_B_TERMS[p][t], I[c]);
      B[p][c] = acc * twelth;
    }
  }
}

static const signed char* hex_terms_of(int p, int j) {
  for (int t = 0; t < 6; ++t)
    if (HEX_B_J[p][t] == j) return HEX_B_TERMS[p][t];
  return NULL; /* unreachable for the tables above */
}

/* geometry.cpp:271-310 get_vol_hex: exact trilinear hex volume. */
double orc_vol_hex(const double x[8], const double y[8], const double z[8]) {
  const double twelth = 1. / 12.;
  double vol = 0.0;
  for (int a = 0; a < 8; ++a) {
    const int i = HEX_V_I[a];
    double inner = y[HEX_V_J[a][0]] * hex_comb(hex_terms_of(i, HEX_V_J[a][0]), z);
    for (int b = 1; b < 6; ++b) inner = inner + y[HEX_V_J[a][b]] * hex_comb(hex_terms_of(i, HEX_V_J[a][b]), z);
    vol = (a == 0) ? x[i] * inner : vol + x[i] * inner;
  }
  return vol * twelth;
}

/* The Mach detector's pow(vol, 1.0/3.0) (force_sgh.cpp:319-320).  The default
 * build calls libm pow, as the reference does.  With -DORC_CR_POW it is the
 * correctly rounded vol^fl(1/3) instead: the exponent is 1/3 - d with
 * d = 2^-54/3, so vol^fl(1/3) = cbrt(vol) (1 - d ln vol + ...); one Newton step on
 * t^3 = vol with an error-free residual plus the -d ln vol term refine cbrt's
 * result to well below an ulp before the final rounding.  glibc's pow is not
 * correctly rounded for about 0.1% of arguments; this variant isolates that
 * libm rounding from the rest of the arithmetic. */
static double orc_pow_third(double v) {
#ifdef ORC_CR_POW
  if (!(v > 1.0e-290 && v < 1.0e290)) return pow(v, 1.0 / 3.0);
  const double c0 = cbrt(v);
  const double p = c0 * c0;
  const double pe = fma(c0, c0, -p);
  const double q = p * c0;
  const double qe = fma(p, c0, -q) + pe * c0;
  const double r = (v - q) - qe;
  const double step = r / (3.0 * p);
  int ex = 0;
  const double m = frexp(v, &ex);
  const double lnv = (double)ex * 0.6931471805599453 + log(m);
  const double lo = step - c0 * (lnv * 1.8503717077085943e-17);
  return c0 + lo;
#else
  return pow(v, 1.0 / 3.0);
#endif
}

/* The CFL distance's pow(d, 2.0) (time_integration.cpp:107-109): libm pow by
 * default, the IEEE square d*d (correctly rounded) with -DORC_CR_POW. */
static double orc_pow2(double d) {
#ifdef ORC_CR_POW
  return d * d;
#else
  return pow(d, 2.0);
#endif
}

/* ------------------------------------------------------------------------- */
struct orc_sim {
  int64_t nn, ne;
  int64_t* nie;              /* [ne][8] */
  /* topology (mesh.h:180-338, setup.cpp:431-665) */
  int64_t* cin_start;        /* corners_in_node CSR [nn+1] */
  int64_t* cin;              /* corner gids, ascending elem (mesh.h:218-241) */
  int64_t* eie_start;        /* elems_in_elem CSR [ne+1] */
  int64_t* eie;
  int nsets;
  int64_t* bset_start;       /* bdy_nodes_in_set CSR [nsets+1] */
  int64_t* bset;
  /* materials / boundaries */
  int nmat, nsv;
  orc_material* mat;
  double* state_vars;
  orc_boundary* bc;
  /* state, reference layouts */
  double *coords, *vel, *node_mass;
  double *den, *pres, *stress, *sspd, *sie, *vol, *div, *mass, *statev;
  int64_t* mat_id;
  double* corner_force;
  /* time control (driver.cpp:35-56) */
  double time_value, dt, graphics_time;
  int64_t cycle;
  int stage;       /* next RK stage within the current cycle, 0 = cycle start */
  int stopped;
};

#define X1(s, n, d) ((s)->coords[(size_t)(s)->nn * 3 + (size_t)(n) * 3 + (d)])
#define X0(s, n, d) ((s)->coords[(size_t)(n) * 3 + (d)])
#define V1(s, n, d) ((s)->vel[(size_t)(s)->nn * 3 + (size_t)(n) * 3 + (d)])
#define V0(s, n, d) ((s)->vel[(size_t)(n) * 3 + (d)])

static void* zalloc(size_t n) {
  void* p = calloc(n ? n : 1, 1);
  return p;
}

static int cmp_i64(const void* a, const void* b) {
  int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
  return (x > y) - (x < y);
}

/* mesh.h:180-245 build_corner_connectivity and mesh.h:249-338
 * build_elem_elem_connectivity (neighbour = any other element sharing a node). */
static void build_topology(orc_sim* s) {
  const int64_t nn = s->nn, ne = s->ne;
  s->cin_start = (int64_t*)zalloc(sizeof(int64_t) * (size_t)(nn + 1));
  for (int64_t e = 0; e < ne; ++e)
    for (int l = 0; l < 8; ++l) s->cin_start[s->nie[e * 8 + l] + 1]++;
  for (int64_t n = 0; n < nn; ++n) s->cin_start[n + 1] += s->cin_start[n];
  s->cin = (int64_t*)zalloc(sizeof(int64_t) * (size_t)(8 * ne));
  int64_t* fill = (int64_t*)zalloc(sizeof(int64_t) * (size_t)nn);
  for (int64_t e = 0; e < ne; ++e)
    for (int l = 0; l < 8; ++l) {
      int64_t n = s->nie[e * 8 + l];
      s->cin[s->cin_start[n] + fill[n]++] = e * 8 + l;
    }
  free(fill);

  s->eie_start = (int64_t*)zalloc(sizeof(int64_t) * (size_t)(ne + 1));
  int64_t* tmp = (int64_t*)zalloc(sizeof(int64_t) * (size_t)ne * 64);
  int64_t* cnt = (int64_t*)zalloc(sizeof(int64_t) * (size_t)ne);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < ne; ++e) {
    int64_t* row = tmp + e * 64;
    int64_t k = 0;
    for (int l = 0; l < 8; ++l) {
      int64_t n = s->nie[e * 8 + l];
      for (int64_t c = s->cin_start[n]; c < s->cin_start[n + 1]; ++c) {
        int64_t nb = s->cin[c] / 8;
        if (nb == e) continue;
        int seen = 0;
        for (int64_t i = 0; i < k; ++i)
          if (row[i] == nb) { seen = 1; break; }
        if (!seen && k < 64) row[k++] = nb;
      }
    }
    cnt[e] = k;
  }
  for (int64_t e = 0; e < ne; ++e) s->eie_start[e + 1] = s->eie_start[e] + cnt[e];
  s->eie = (int64_t*)zalloc(sizeof(int64_t) * (size_t)s->eie_start[ne]);
  for (int64_t e = 0; e < ne; ++e)
    memcpy(s->eie + s->eie_start[e], tmp + e * 64, sizeof(int64_t) * (size_t)cnt[e]);
  free(tmp);
  free(cnt);
}

orc_sim* orc_create(int64_t num_nodes, int64_t num_elems, const int64_t* nodes_in_elem,
                    const double* coords) {
  if (num_nodes <= 0 || num_elems <= 0 || !nodes_in_elem || !coords) return NULL;
  for (int64_t i = 0; i < num_elems * 8; ++i)
    if (nodes_in_elem[i] < 0 || nodes_in_elem[i] >= num_nodes) return NULL;
  orc_sim* s = (orc_sim*)zalloc(sizeof(orc_sim));
  s->nn = num_nodes;
  s->ne = num_elems;
  size_t nn = (size_t)num_nodes, ne = (size_t)num_elems;
  s->nie = (int64_t*)zalloc(sizeof(int64_t) * ne * 8);
  memcpy(s->nie, nodes_in_elem, sizeof(int64_t) * ne * 8);
  s->coords = (double*)zalloc(sizeof(double) * 2 * nn * 3);
  s->vel = (double*)zalloc(sizeof(double) * 2 * nn * 3);
  s->node_mass = (double*)zalloc(sizeof(double) * nn);
  /* read_mesh.cpp:61-135: coordinates land in bin 0 and are copied to bin 1. */
  memcpy(s->coords, coords, sizeof(double) * nn * 3);
  memcpy(s->coords + nn * 3, coords, sizeof(double) * nn * 3);
  s->den = (double*)zalloc(sizeof(double) * ne);
  s->pres = (double*)zalloc(sizeof(double) * ne);
  s->stress = (double*)zalloc(sizeof(double) * 2 * ne * 9);
  s->sspd = (double*)zalloc(sizeof(double) * ne);
  s->sie = (double*)zalloc(sizeof(double) * 2 * ne);
  s->vol = (double*)zalloc(sizeof(double) * ne);
  s->div = (double*)zalloc(sizeof(double) * ne);
  s->mass = (double*)zalloc(sizeof(double) * ne);
  s->mat_id = (int64_t*)zalloc(sizeof(int64_t) * ne);
  s->corner_force = (double*)zalloc(sizeof(double) * ne * 24);
  build_topology(s);
  return s;
}

void orc_destroy(orc_sim* s) {
  if (!s) return;
  free(s->nie); free(s->cin_start); free(s->cin); free(s->eie_start); free(s->eie);
  free(s->bset_start); free(s->bset); free(s->mat); free(s->state_vars); free(s->bc);
  free(s->coords); free(s->vel); free(s->node_mass); free(s->den); free(s->pres);
  free(s->stress); free(s->sspd); free(s->sie); free(s->vol); free(s->div); free(s->mass);
  free(s->statev); free(s->mat_id); free(s->corner_force);
  free(s);
}

int orc_set_materials(orc_sim* s, int num_materials, const orc_material* m, int num_state_vars,
                      const double* state_vars) {
  if (num_materials <= 0 || num_state_vars < 2) return 1;
  for (int i = 0; i < num_materials; ++i) {
    if (m[i].eos_model != 0 || m[i].strength_type < 0 || m[i].strength_type > 2) return 1;
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

int orc_set_boundaries(orc_sim* s, int num_bcs, const orc_boundary* b) {
  if (num_bcs < 0) return 1;
  for (int i = 0; i < num_bcs; ++i) {
    if (b[i].hydro_bc < 0 || b[i].hydro_bc > 5) return 1; /* bdy_hydro_conds, mesh.h:910-918 */
    if (b[i].hydro_bc == 1 && (b[i].surface < 0 || b[i].surface > 2)) return 1;
    if (b[i].surface < 0 || b[i].surface > 4) return 1;
  }
  free(s->bc);
  s->nsets = num_bcs;
  s->bc = (orc_boundary*)zalloc(sizeof(orc_boundary) * (size_t)(num_bcs ? num_bcs : 1));
  if (num_bcs) memcpy(s->bc, b, sizeof(orc_boundary) * (size_t)num_bcs);
  return 0;
}

/* setup.cpp:487-571 check_bdy on one patch: all its nodes within 1e-7 of the surface. */
static int patch_on_surface(const orc_sim* s, const int64_t* pn, int tag, double val) {
  int on = 0;
  for (int k = 0; k < 4; ++k) {
    double c0 = X1(s, pn[k], 0), c1 = X1(s, pn[k], 1), c2 = X1(s, pn[k], 2);
    if (tag == 0) { if (fabs(c0 - val) <= 1.0e-7) on += 1; }
    else if (tag == 1) { if (fabs(c1 - val) <= 1.0e-7) on += 1; }
    else if (tag == 2) { if (fabs(c2 - val) <= 1.0e-7) on += 1; }
    else if (tag == 3) { double R = sqrt(c0 * c0 + c1 * c1); if (fabs(R - val) <= 1.0e-7) on += 1; }
    else if (tag == 4) { double R = sqrt(c0 * c0 + c1 * c1 + c2 * c2); if (fabs(R - val) <= 1.0e-7) on += 1; }
  }
  return on == 4;
}

typedef struct { int64_t key[4]; int64_t elem; int patch; } face_rec;
static int cmp_face(const void* a, const void* b) {
  const face_rec* x = (const face_rec*)a;
  const face_rec* y = (const face_rec*)b;
  for (int i = 0; i < 4; ++i)
    if (x->key[i] != y->key[i]) return (x->key[i] > y->key[i]) - (x->key[i] < y->key[i]);
  return 0;
}

/* mesh.h:342-649 boundary patches (faces owned by one element), then
 * setup.cpp:431-480 tag_bdys and setup.cpp:575-665 build_boundry_node_sets. */
static void build_bdy_sets(orc_sim* s) {
  const int64_t ne = s->ne;
  face_rec* f = (face_rec*)zalloc(sizeof(face_rec) * (size_t)ne * 6);
  for (int64_t e = 0; e < ne; ++e)
    for (int p = 0; p < 6; ++p) {
      face_rec* r = &f[e * 6 + p];
      for (int k = 0; k < 4; ++k) r->key[k] = s->nie[e * 8 + HEX_PATCH[p][k]];
      qsort(r->key, 4, sizeof(int64_t), cmp_i64);
      r->elem = e;
      r->patch = p;
    }
  qsort(f, (size_t)ne * 6, sizeof(face_rec), cmp_face);
  char* is_bdy_node_in = (char*)zalloc((size_t)s->nn * (size_t)(s->nsets ? s->nsets : 1));
  for (int64_t i = 0; i < ne * 6;) {
    int64_t j = i + 1;
    while (j < ne * 6 && cmp_face(&f[i], &f[j]) == 0) ++j;
    if (j - i == 1) {
      int64_t pn[4];
      for (int k = 0; k < 4; ++k) pn[k] = s->nie[f[i].elem * 8 + HEX_PATCH[f[i].patch][k]];
      for (int b = 0; b < s->nsets; ++b)
        if (patch_on_surface(s, pn, s->bc[b].surface, s->bc[b].value))
          for (int k = 0; k < 4; ++k) is_bdy_node_in[(size_t)b * (size_t)s->nn + (size_t)pn[k]] = 1;
    }
    i = j;
  }
  free(f);
  free(s->bset_start); free(s->bset);
  s->bset_start = (int64_t*)zalloc(sizeof(int64_t) * (size_t)(s->nsets + 1));
  int64_t total = 0;
  for (int b = 0; b < s->nsets; ++b)
    for (int64_t n = 0; n < s->nn; ++n) total += is_bdy_node_in[(size_t)b * (size_t)s->nn + (size_t)n];
  s->bset = (int64_t*)zalloc(sizeof(int64_t) * (size_t)(total ? total : 1));
  int64_t k = 0;
  for (int b = 0; b < s->nsets; ++b) {
    for (int64_t n = 0; n < s->nn; ++n)
      if (is_bdy_node_in[(size_t)b * (size_t)s->nn + (size_t)n]) s->bset[k++] = n;
    s->bset_start[b + 1] = k;
  }
  free(is_bdy_node_in);
}

static void gather_x1(const orc_sim* s, int64_t e, double x[8], double y[8], double z[8]) {
  for (int l = 0; l < 8; ++l) {
    int64_t n = s->nie[e * 8 + l];
    x[l] = X1(s, n, 0);
    y[l] = X1(s, n, 1);
    z[l] = X1(s, n, 2);
  }
}

/* geometry.cpp:238-267 get_vol */
static void get_vol(orc_sim* s) {
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < s->ne; ++e) {
    double x[8], y[8], z[8];
    gather_x1(s, e, x, y, z);
    s->vol[e] = orc_vol_hex(x, y, z);
  }
}

/* eos.cpp:12-46 ideal_gas */
static void ideal_gas(orc_sim* s, int64_t e, double den, double sie) {
  double gamma = s->statev[e * s->nsv + 0];
  double csmin = s->statev[e * s->nsv + 1];
  s->pres[e] = (gamma - 1.0) * sie * den;
  s->sspd[e] = sqrt(gamma * (gamma - 1.0) * sie);
  if (s->sspd[e] < csmin) s->sspd[e] = csmin;
}

/* boundary.cpp:10-55 boundary_velocity */
static void boundary_velocity(orc_sim* s) {
  for (int b = 0; b < s->nsets; ++b) {
    for (int64_t k = s->bset_start[b]; k < s->bset_start[b + 1]; ++k) {
      int64_t n = s->bset[k];
      if (s->bc[b].hydro_bc == 1) {
        V1(s, n, s->bc[b].surface) = 0.0;
      } else if (s->bc[b].hydro_bc == 0) {
        for (int d = 0; d < 3; ++d) V1(s, n, d) = 0.0;
      }
    }
  }
}

int orc_setup(orc_sim* s, int num_fills, const orc_fill* fills) {
  if (!s->mat || (s->nsets > 0 && !s->bc)) return 1;
  for (int f = 0; f < num_fills; ++f)
    if (fills[f].mat_id < 0 || fills[f].mat_id >= s->nmat) return 1;
  get_vol(s);        /* driver.cpp:239 */
  build_bdy_sets(s); /* setup.cpp:37-43 */
  const int64_t ne = s->ne;
  const double PI = 3.141592653589793;
  for (int f = 0; f < num_fills; ++f) { /* setup.cpp:109-357 */
    const orc_fill* F = &fills[f];
    for (int64_t e = 0; e < ne; ++e) {
      double ec[3] = {0.0, 0.0, 0.0};
      for (int l = 0; l < 8; ++l) {
        int64_t n = s->nie[e * 8 + l];
        ec[0] += X1(s, n, 0);
        ec[1] += X1(s, n, 1);
        ec[2] += X1(s, n, 2);
      }
      ec[0] = ec[0] / 8;
      ec[1] = ec[1] / 8;
      ec[2] = ec[2] / 8;
      double radius = sqrt(ec[0] * ec[0] + ec[1] * ec[1] + ec[2] * ec[2]);
      double radius_cyl = sqrt(ec[0] * ec[0] + ec[1] * ec[1]);
      int fill_this = 0;
      switch (F->volume) {
        case 0: fill_this = 1; break;
        case 1:
          if (ec[0] >= F->x1 && ec[0] <= F->x2 && ec[1] >= F->y1 && ec[1] <= F->y2 &&
              ec[2] >= F->z1 && ec[2] <= F->z2)
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
      for (int l = 0; l < 8; ++l) {
        int64_t n = s->nie[e * 8 + l];
        if (F->velocity == 0) {
          V1(s, n, 0) = F->u;
          V1(s, n, 1) = F->v;
          V1(s, n, 2) = F->w;
        } else if (F->velocity == 1 || F->velocity == 2) {
          const int nd = (F->velocity == 1) ? 2 : 3;
          double dir[3] = {0.0, 0.0, 0.0};
          double radius_val = 0.0;
          for (int d = 0; d < nd; ++d) {
            dir[d] = X1(s, n, d);
            radius_val += X1(s, n, d) * X1(s, n, d);
          }
          radius_val = sqrt(radius_val);
          for (int d = 0; d < nd; ++d) {
            if (radius_val > 1.0e-14) dir[d] /= (radius_val);
            else dir[d] = 0.0;
          }
          V1(s, n, 0) = F->speed * dir[0];
          V1(s, n, 1) = F->speed * dir[1];
          V1(s, n, 2) = (nd == 3) ? F->speed * dir[2] : 0.0;
        } else if (F->velocity == 5) {
          V1(s, n, 0) = sin(PI * X1(s, n, 0)) * cos(PI * X1(s, n, 1));
          V1(s, n, 1) = -1.0 * cos(PI * X1(s, n, 0)) * sin(PI * X1(s, n, 1));
          V1(s, n, 2) = 0.0;
        }
      }
      if (F->velocity == 5) {
        s->pres[e] = 0.25 * (cos(2.0 * PI * ec[0]) + cos(2.0 * PI * ec[1])) + 1.0;
        double gamma = s->statev[e * s->nsv + 4];
        s->sie[ne + e] = s->pres[e] / (F->den * (gamma - 1.0));
      }
    }
  }
  boundary_velocity(s); /* setup.cpp:362 */
  /* setup.cpp:394-420 node mass: sum over elems_in_node (corner order). */
  for (int64_t n = 0; n < s->nn; ++n) {
    double m = 0.0;
    for (int64_t c = s->cin_start[n]; c < s->cin_start[n + 1]; ++c)
      m += 1.0 / 8.0 * s->mass[s->cin[c] / 8];
    s->node_mass[n] = m;
  }
  return 0;
}

void orc_init_time(orc_sim* s, const orc_params* p) {
  s->time_value = 0.0;
  s->dt = p->dt_start;
  s->graphics_time = p->graphics_dt_ival;
  s->cycle = 0;
  s->stage = 0;
  s->stopped = 0;
}

/* time_integration.cpp:54-154 get_timestep (3D). */
static void get_timestep(orc_sim* s, const orc_params* p) {
  s->dt = s->dt * 1.1;
  double min_dt_calc = 1.7976931348623157e308;
#pragma omp parallel
  {
    double lcl = 1.7976931348623157e308;
#pragma omp for schedule(static)
    for (int64_t e = 0; e < s->ne; ++e) {
      double c[8][3];
      for (int l = 0; l < 8; ++l)
        for (int d = 0; d < 3; ++d) c[l][d] = X1(s, s->nie[e * 8 + l], d);
      double dist[28];
      int a = 0, b = 1, loop = 0;
      for (int i = 0; i < 28; ++i) {
        dist[i] = fabs(sqrt(orc_pow2(c[b][0] - c[a][0]) + orc_pow2(c[b][1] - c[a][1]) +
                            orc_pow2(c[b][2] - c[a][2])));
        b++;
        a++;
        if (b > 7) {
          loop++;
          b = 1 + loop;
          a = 0;
        }
      }
      double dist_min = dist[0];
      for (int i = 0; i < 28; ++i) dist_min = fmin(dist[i], dist_min);
      double dt_l = p->dt_cfl * dist_min / (s->sspd[e] + p->fuzz);
      dt_l = fmin(dt_l, p->dt_max);
      dt_l = fmax(dt_l, p->dt_min);
      if (dt_l < lcl) lcl = dt_l;
    }
#pragma omp critical(orc_dt)
    if (lcl < min_dt_calc) min_dt_calc = lcl;
  }
  if (min_dt_calc < s->dt) s->dt = min_dt_calc;
  s->dt = fmin(s->dt, (s->graphics_time - s->time_value) + p->fuzz);
  s->dt = fmin(s->dt, p->time_final - s->time_value);
}

/* time_integration.cpp:9-44 rk_init */
static void rk_init(orc_sim* s) {
  const size_t nn = (size_t)s->nn, ne = (size_t)s->ne;
  memcpy(s->stress, s->stress + ne * 9, sizeof(double) * ne * 9);
  memcpy(s->sie, s->sie + ne, sizeof(double) * ne);
  memcpy(s->coords, s->coords + nn * 3, sizeof(double) * nn * 3);
  memcpy(s->vel, s->vel + nn * 3, sizeof(double) * nn * 3);
}

/* momentum.cpp:221-292 get_divergence */
static void get_divergence(orc_sim* s) {
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < s->ne; ++e) {
    double x[8], y[8], z[8], B[8][3], u[8], v[8], w[8];
    gather_x1(s, e, x, y, z);
    orc_bmatrix(x, y, z, B);
    for (int l = 0; l < 8; ++l) {
      int64_t n = s->nie[e * 8 + l];
      u[l] = V1(s, n, 0);
      v[l] = V1(s, n, 1);
      w[l] = V1(s, n, 2);
    }
    double inverse_vol = 1.0 / s->vol[e];
    double d = 0.0;
    double sx = u[0] * B[0][0], sy = v[0] * B[0][1], sz = w[0] * B[0][2];
    for (int l = 1; l < 8; ++l) {
      sx = sx + u[l] * B[l][0];
      sy = sy + v[l] * B[l][1];
      sz = sz + w[l] * B[l][2];
    }
    d += sx * inverse_vol;
    d += sy * inverse_vol;
    d += sz * inverse_vol;
    s->div[e] = d;
  }
}

/* momentum.cpp:59-144 get_velgrad: L(i,j) = (sum_l v_i(l) B(l,j)) / vol with B the
 * outward corner normals, summed over l in order, times the reciprocal volume. */
static void get_velgrad(double L[3][3], const double u[8], const double v[8], const double w[8],
                        double B[8][3], double vol) {
  const double inverse_vol = 1.0 / vol;
  const double* vc[3] = {u, v, w};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double acc = vc[i][0] * B[0][j];
      for (int l = 1; l < 8; ++l) acc = acc + vc[i][l] * B[l][j];
      L[i][j] = acc * inverse_vol;
    }
}

/* The test strength model the reference oracle build assigns through
 * material_t::strength_model (oracle/ref/ref_user_mat.cpp): linear
 * hypo-elasticity of the deviatoric stress, G = statev(3),
 * stress(1) = stress(0) + rk_alpha dt 2 G (D - tr(D)/3 I), D = (L + L^T)/2. */
static void strength_model(orc_sim* s, int64_t e, double L[3][3], double dt, double rk_alpha) {
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

/* force_sgh.cpp:12-399 get_force_sgh (3D).  The shock direction and curl terms
 * of the reference feed only unused variables (use_shock_dir = 0 at :227,
 * phi_curl unused at :331) and are omitted; the velocity gradient is formed for
 * hypo materials only, whose strength model (:366-391) reads it. */
static void get_force_sgh(orc_sim* s, const orc_params* p, double rk_alpha) {
  const double fuzz = p->fuzz, small = p->small;
  const size_t ne = (size_t)s->ne;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < s->ne; ++e) {
    double x[8], y[8], z[8], an[8][3], tau[3][3], muc[8], sum[4], vel_star[3];
    double vol = s->vol[e];
    double Bout[8][3];
    gather_x1(s, e, x, y, z);
    orc_bmatrix(x, y, z, an);
    memcpy(Bout, an, sizeof(Bout));
    for (int l = 0; l < 8; ++l)
      for (int d = 0; d < 3; ++d) an[l][d] = (-1.0) * an[l][d];
    double div = s->div[e];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) tau[i][j] = s->stress[ne * 9 + (size_t)e * 9 + (size_t)(i * 3 + j)];
    for (int i = 0; i < 3; ++i) tau[i][i] -= s->pres[e];
    for (int d = 0; d < 3; ++d) vel_star[d] = 0.0;
    for (int l = 0; l < 8; ++l) {
      int64_t n = s->nie[e * 8 + l];
      vel_star[0] += 0.125 * V1(s, n, 0);
      vel_star[1] += 0.125 * V1(s, n, 1);
      vel_star[2] += 0.125 * V1(s, n, 2);
    }
    for (int i = 0; i < 4; ++i) sum[i] = 0.0;
    const orc_material* M = &s->mat[s->mat_id[e]];
    for (int l = 0; l < 8; ++l) {
      int64_t n = s->nie[e * 8 + l];
      double v0 = V1(s, n, 0), v1 = V1(s, n, 1), v2 = V1(s, n, 2);
      double mag_vel = sqrt((v0 - vel_star[0]) * (v0 - vel_star[0]) +
                            (v1 - vel_star[1]) * (v1 - vel_star[1]) +
                            (v2 - vel_star[2]) * (v2 - vel_star[2]));
      if (div < 0) muc[l] = s->den[e] * (M->q1 * s->sspd[e] + M->q2 * mag_vel);
      else muc[l] = s->den[e] * (M->q1ex * s->sspd[e] + M->q2ex * mag_vel);
      double mu_term = muc[l] * sqrt(an[l][0] * an[l][0] + an[l][1] * an[l][1] + an[l][2] * an[l][2]);
      sum[0] += mu_term * v0;
      sum[1] += mu_term * v1;
      sum[2] += mu_term * v2;
      sum[3] += mu_term;
      muc[l] = mu_term;
    }
    if (sum[3] > fuzz) {
      for (int i = 0; i < 3; ++i) vel_star[i] = sum[i] / sum[3];
    } else {
      for (int i = 0; i < 3; ++i) vel_star[i] = 0.0;
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
    double c_length = orc_pow_third(vol);
    double alpha = fmin(1.0, omega * (c_length * fabs(div)) / (s->sspd[e] + fuzz));
    phi = alpha * phi;
    for (int l = 0; l < 8; ++l) {
      int64_t n = s->nie[e * 8 + l];
      for (int d = 0; d < 3; ++d) {
        s->corner_force[((size_t)e * 8 + (size_t)l) * 3 + (size_t)d] =
            an[l][0] * tau[0][d] + an[l][1] * tau[1][d] + an[l][2] * tau[2][d] +
            phi * muc[l] * (vel_star[d] - V1(s, n, d));
      }
    }
    if (M->strength_type == 1) {
      double u[8], v[8], w[8], L[3][3];
      for (int l = 0; l < 8; ++l) {
        int64_t n = s->nie[e * 8 + l];
        u[l] = V1(s, n, 0);
        v[l] = V1(s, n, 1);
        w[l] = V1(s, n, 2);
      }
      get_velgrad(L, u, v, w, Bout, vol);
      strength_model(s, e, L, s->dt, rk_alpha);
    }
  }
}

/* momentum.cpp:11-53 update_velocity_sgh */
static void update_velocity(orc_sim* s, double rk_alpha, double dt) {
#pragma omp parallel for schedule(static)
  for (int64_t n = 0; n < s->nn; ++n) {
    double F[3] = {0.0, 0.0, 0.0};
    for (int64_t c = s->cin_start[n]; c < s->cin_start[n + 1]; ++c)
      for (int d = 0; d < 3; ++d) F[d] += s->corner_force[(size_t)s->cin[c] * 3 + (size_t)d];
    for (int d = 0; d < 3; ++d) V1(s, n, d) = V0(s, n, d) + rk_alpha * dt * F[d] / s->node_mass[n];
  }
}

/* energy_sgh.cpp:6-55 update_energy_sgh (3D: node_radius = 1) */
static void update_energy(orc_sim* s, double rk_alpha, double dt) {
  const size_t ne = (size_t)s->ne;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < s->ne; ++e) {
    double elem_power = 0.0;
    for (int l = 0; l < 8; ++l) {
      int64_t n = s->nie[e * 8 + l];
      double node_radius = 1;
      for (int d = 0; d < 3; ++d) {
        double half_vel = (V1(s, n, d) + V0(s, n, d)) * 0.5;
        elem_power += s->corner_force[((size_t)e * 8 + (size_t)l) * 3 + (size_t)d] * node_radius * half_vel;
      }
    }
    s->sie[ne + (size_t)e] = s->sie[e] - rk_alpha * dt / s->mass[e] * elem_power;
  }
}

/* geometry.cpp:9-26 update_position_sgh */
static void update_position(orc_sim* s, double rk_alpha, double dt) {
#pragma omp parallel for schedule(static)
  for (int64_t n = 0; n < s->nn; ++n)
    for (int d = 0; d < 3; ++d) {
      double half_vel = (V1(s, n, d) + V0(s, n, d)) * 0.5;
      X1(s, n, d) = X0(s, n, d) + rk_alpha * dt * half_vel;
    }
}

/* properties.cpp:9-114 update_state: density, the hyper strength model with the
 * velocity gradient of the updated state (:46-95), then the EOS. */
static void update_state(orc_sim* s, double rk_alpha) {
  const size_t ne = (size_t)s->ne;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < s->ne; ++e) {
    s->den[e] = s->mass[e] / s->vol[e];
    if (s->mat[s->mat_id[e]].strength_type == 2) {
      double x[8], y[8], z[8], B[8][3], u[8], v[8], w[8], L[3][3];
      gather_x1(s, e, x, y, z);
      orc_bmatrix(x, y, z, B);
      for (int l = 0; l < 8; ++l) {
        int64_t n = s->nie[e * 8 + l];
        u[l] = V1(s, n, 0);
        v[l] = V1(s, n, 1);
        w[l] = V1(s, n, 2);
      }
      get_velgrad(L, u, v, w, B, s->vol[e]);
      strength_model(s, e, L, s->dt, rk_alpha);
    }
    ideal_gas(s, e, s->den[e], s->sie[ne + (size_t)e]);
  }
}

/* One RK stage (sgh_solve.cpp:349-585). */
static void rk_stage(orc_sim* s, const orc_params* p, int stage) {
  double rk_alpha = 1.0 / ((double)p->rk_num_stages - (double)stage);
  get_divergence(s);
  get_force_sgh(s, p, rk_alpha);
  update_velocity(s, rk_alpha, s->dt);
  boundary_velocity(s);
  update_energy(s, rk_alpha, s->dt);
  update_position(s, rk_alpha, s->dt);
  get_vol(s);
  update_state(s, rk_alpha);
}

/* sgh_solve.cpp:590-632: time advance, graphics-time bookkeeping, stop test. */
static void end_cycle(orc_sim* s, const orc_params* p) {
  s->time_value += s->dt;
  int write = 0;
  if ((s->cycle + 1) % p->graphics_cyc_ival == 0 && s->cycle > 0) write = 1;
  else if (s->time_value >= p->time_final) write = 1;
  else if (s->time_value >= s->graphics_time) write = 1;
  if (write) s->graphics_time = s->time_value + p->graphics_dt_ival;
  if (s->time_value >= p->time_final) s->stopped = 1;
  s->cycle++;
}

int64_t orc_run_stages(orc_sim* s, const orc_params* p, int64_t nstages) {
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

int64_t orc_run_cycles(orc_sim* s, const orc_params* p, int64_t ncycles) {
  int64_t c0 = s->cycle;
  for (int64_t c = 0; c < ncycles && !s->stopped; ++c) orc_run_stages(s, p, p->rk_num_stages - s->stage);
  return s->cycle - c0;
}

void orc_energy(const orc_sim* s, double* ie, double* ke) {
  double IE = 0.0, KE = 0.0;
  for (int64_t e = 0; e < s->ne; ++e) IE += s->mass[e] * s->sie[(size_t)s->ne + (size_t)e];
  for (int64_t n = 0; n < s->nn; ++n) {
    double k = 0;
    for (int d = 0; d < 3; ++d) k += V1(s, n, d) * V1(s, n, d);
    KE += s->node_mass[n] * k;
  }
  if (ie) *ie = IE;
  if (ke) *ke = 0.5 * KE;
}

void orc_time(const orc_sim* s, double* time_value, double* dt, double* graphics_time, int64_t* cycle) {
  if (time_value) *time_value = s->time_value;
  if (dt) *dt = s->dt;
  if (graphics_time) *graphics_time = s->graphics_time;
  if (cycle) *cycle = s->cycle;
}

static int64_t array_info(const orc_sim* s, int which, void** ptr, size_t* esize) {
  const int64_t nn = s->nn, ne = s->ne;
  *esize = sizeof(double);
  switch (which) {
    case ORC_NODE_COORDS: *ptr = s->coords; return 2 * nn * 3;
    case ORC_NODE_VEL: *ptr = s->vel; return 2 * nn * 3;
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
    case ORC_ELEM_STATEV: *ptr = s->statev; return s->statev ? ne * s->nsv : 0;
    case ORC_CORNER_FORCE: *ptr = s->corner_force; return ne * 24;
    default: *ptr = NULL; return -1;
  }
}

int64_t orc_get(const orc_sim* s, int which, void* out) {
  if (which == ORC_BDY_NODE_MASK) {
    /* per node: bit d set when some boundary set zeroes velocity component d */
    int32_t* m = (int32_t*)out;
    memset(m, 0, sizeof(int32_t) * (size_t)s->nn);
    for (int b = 0; b < s->nsets; ++b)
      for (int64_t k = s->bset_start[b]; k < s->bset_start[b + 1]; ++k)
        m[s->bset[k]] |= s->bc[b].hydro_bc == 1 ? (1 << s->bc[b].surface) : s->bc[b].hydro_bc == 0 ? 7 : 0;
    return s->nn;
  }
  void* p;
  size_t es;
  int64_t n = array_info(s, which, &p, &es);
  if (n < 0) return -1;
  if (out && p) memcpy(out, p, es * (size_t)n);
  return n;
}

int64_t orc_set(orc_sim* s, int which, const void* in) {
  void* p;
  size_t es;
  int64_t n = array_info(s, which, &p, &es);
  if (n < 0 || !p) return -1;
  memcpy(p, in, es * (size_t)n);
  return n;
}
