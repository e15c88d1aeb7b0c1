// Host side of libfierro_sgh: errors, mesh validation and topology (corner and
// neighbour CSR, boundary node sets, Morton renumbering) and the set-up of the
// initial state (setup.cpp:10-424).  Compiled with -ffp-contract=off so the
// set-up doubles follow the reference's uncontracted evaluation.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "fierro_sgh.h"
#include "sgh_hex.h"
#include "sgh_internal.h"
#include "sgh_rz.h"
#include "sgh_setup.h"

namespace fierro {

static thread_local std::string g_err;

int set_error(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

void clear_error() { g_err.clear(); }

namespace {

// Node -> element CSR in the caller's numbering, elements ascending per node
// (the corner order of build_corner_connectivity, mesh.h:218-241).
void node_elem_csr(int64_t nn, int64_t ne, const uint64_t* nie, std::vector<int64_t>* start,
                   std::vector<int64_t>* elems, std::vector<int8_t>* lids) {
  start->assign((size_t)nn + 1, 0);
  for (int64_t i = 0; i < ne * 8; ++i) (*start)[nie[i] + 1]++;
  for (int64_t n = 0; n < nn; ++n) (*start)[n + 1] += (*start)[n];
  elems->resize((size_t)ne * 8);
  if (lids) lids->resize((size_t)ne * 8);
  std::vector<int64_t> fill(start->begin(), start->end() - 1);
  for (int64_t e = 0; e < ne; ++e)
    for (int l = 0; l < 8; ++l) {
      int64_t n = (int64_t)nie[e * 8 + l];
      int64_t k = fill[n]++;
      (*elems)[k] = e;
      if (lids) (*lids)[k] = (int8_t)l;
    }
}

bool elem_has_node(const uint64_t* nie, int64_t e, uint64_t n) {
  for (int l = 0; l < 8; ++l)
    if (nie[e * 8 + l] == n) return true;
  return false;
}

// check_bdy (setup.cpp:487-571) for one node of a patch.
bool node_on_surface(const double* c, int tag, double val) {
  if (tag == 0) return std::fabs(c[0] - val) <= 1.0e-7;
  if (tag == 1) return std::fabs(c[1] - val) <= 1.0e-7;
  if (tag == 2) return std::fabs(c[2] - val) <= 1.0e-7;
  if (tag == 3) return std::fabs(std::sqrt(c[0] * c[0] + c[1] * c[1]) - val) <= 1.0e-7;
  if (tag == 4) return std::fabs(std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]) - val) <= 1.0e-7;
  return false;
}

uint64_t spread21(uint64_t v) {
  v &= 0x1FFFFF;
  v = (v | (v << 32)) & 0x1F00000000FFFFULL;
  v = (v | (v << 16)) & 0x1F0000FF0000FFULL;
  v = (v | (v << 8)) & 0x100F00F00F00F00FULL;
  v = (v | (v << 4)) & 0x10C30C30C30C30C3ULL;
  v = (v | (v << 2)) & 0x1249249249249249ULL;
  return v;
}

// Stable LSD radix sort of indices by 63-bit keys (16-bit digits).
std::vector<int64_t> radix_order(const std::vector<uint64_t>& key) {
  const size_t n = key.size();
  std::vector<int64_t> idx(n), tmp(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::vector<size_t> cnt(65537);
  for (int pass = 0; pass < 4; ++pass) {
    const int sh = pass * 16;
    std::fill(cnt.begin(), cnt.end(), 0);
    for (size_t i = 0; i < n; ++i) cnt[((key[idx[i]] >> sh) & 0xFFFF) + 1]++;
    for (size_t d = 0; d < 65536; ++d) cnt[d + 1] += cnt[d];
    for (size_t i = 0; i < n; ++i) tmp[cnt[(key[idx[i]] >> sh) & 0xFFFF]++] = idx[i];
    idx.swap(tmp);
  }
  return idx;
}

// Morton keys of points, quantised on the bounding box to 21 bits per axis.
std::vector<uint64_t> morton_keys(const double* pts, int64_t n) {
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int64_t i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], pts[i * 3 + d]);
      hi[d] = std::max(hi[d], pts[i * 3 + d]);
    }
  std::vector<uint64_t> key((size_t)n);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    uint64_t q[3];
    for (int d = 0; d < 3; ++d) {
      double span = hi[d] - lo[d];
      double f = span > 0 ? (pts[i * 3 + d] - lo[d]) / span : 0.0;
      q[d] = (uint64_t)std::min(2097151.0, std::max(0.0, f * 2097151.0));
    }
    key[i] = spread21(q[0]) | (spread21(q[1]) << 1) | (spread21(q[2]) << 2);
  }
  return key;
}

}  // namespace

std::vector<int64_t> morton_order(const double* pts, int64_t n) { return radix_order(morton_keys(pts, n)); }

int boundary_masks(const fierro_mesh* mesh, const fierro_boundary* bcs, int64_t num_bcs,
                   const double* coords, std::vector<uint8_t>* mask_ext,
                   std::vector<std::vector<int64_t>>* set_nodes) {
  const int64_t nn = mesh->num_nodes, ne = mesh->num_elems;
  const uint64_t* nie = mesh->nodes_in_elem;
  std::vector<int64_t> start, elems;
  node_elem_csr(nn, ne, nie, &start, &elems, nullptr);
  // boundary patches: faces whose four nodes no other element shares (mesh.h:501-515)
  int nthreads = 1;
#ifdef _OPENMP
  nthreads = omp_get_max_threads();
#endif
  std::vector<std::vector<int64_t>> found((size_t)nthreads);
#pragma omp parallel
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    auto& out = found[(size_t)tid];
#pragma omp for schedule(static)
    for (int64_t e = 0; e < ne; ++e) {
      for (int f = 0; f < 6; ++f) {
        uint64_t a = nie[e * 8 + hex::PATCH[f][0]];
        uint64_t b = nie[e * 8 + hex::PATCH[f][1]];
        uint64_t c = nie[e * 8 + hex::PATCH[f][2]];
        uint64_t d = nie[e * 8 + hex::PATCH[f][3]];
        bool shared = false;
        for (int64_t k = start[a]; k < start[a + 1] && !shared; ++k) {
          int64_t o = elems[k];
          if (o != e && elem_has_node(nie, o, b) && elem_has_node(nie, o, c) && elem_has_node(nie, o, d))
            shared = true;
        }
        if (!shared) out.push_back(e * 6 + f);
      }
    }
  }
  mask_ext->assign((size_t)nn, 0);
  if (set_nodes) set_nodes->assign((size_t)num_bcs, {});
  std::vector<char> in_set((size_t)nn);
  for (int64_t s = 0; s < num_bcs; ++s) {
    std::fill(in_set.begin(), in_set.end(), 0);
    for (auto& v : found)
      for (int64_t pf : v) {
        int64_t e = pf / 6;
        int f = (int)(pf % 6);
        bool all = true;
        for (int k = 0; k < 4 && all; ++k)
          all = node_on_surface(coords + nie[e * 8 + hex::PATCH[f][k]] * 3, bcs[s].surface, bcs[s].value);
        if (all)
          for (int k = 0; k < 4; ++k) in_set[nie[e * 8 + hex::PATCH[f][k]]] = 1;
      }
    uint8_t bits = bc_mask_bits(bcs[s].hydro_bc, bcs[s].surface, 3);
    for (int64_t n = 0; n < nn; ++n)
      if (in_set[n]) {
        (*mask_ext)[n] |= bits;
        if (set_nodes) (*set_nodes)[s].push_back(n);
      }
  }
  return FIERRO_OK;
}

int check_mesh_header(const fierro_mesh* m) {
  if (!m) return set_error(FIERRO_EINVAL, "mesh is NULL");
  if (m->num_dims != 0 && m->num_dims != 2 && m->num_dims != 3)
    return set_error(FIERRO_EINVAL, "mesh num_dims %lld: 3 (hex) or 2 (2D-RZ quads)", (long long)m->num_dims);
  const int npe = mesh_dims(m) == 2 ? 4 : 8;
  if (m->num_nodes < npe || m->num_elems < 1)
    return set_error(FIERRO_EINVAL, "mesh needs at least one element (num_nodes=%lld num_elems=%lld)",
                     (long long)m->num_nodes, (long long)m->num_elems);
  if (!m->nodes_in_elem || !m->coords) return set_error(FIERRO_EINVAL, "mesh arrays are NULL");
  if (m->num_elems * npe >= (int64_t)INT32_MAX || m->num_nodes >= (int64_t)INT32_MAX)
    return set_error(FIERRO_EINVAL, "mesh too large for 32-bit device indices");
  return FIERRO_OK;
}

static int validate_mesh(const fierro_mesh* m) {
  int rc = check_mesh_header(m);
  if (rc) return rc;
  for (int64_t e = 0; e < m->num_elems; ++e) {
    for (int l = 0; l < 8; ++l) {
      uint64_t n = m->nodes_in_elem[e * 8 + l];
      if (n >= (uint64_t)m->num_nodes)
        return set_error(FIERRO_EINVAL, "element %lld node %d id %llu out of range", (long long)e, l,
                         (unsigned long long)n);
      for (int k = 0; k < l; ++k)
        if (m->nodes_in_elem[e * 8 + k] == n)
          return set_error(FIERRO_EINVAL, "element %lld repeats node %llu", (long long)e, (unsigned long long)n);
    }
  }
  for (int64_t i = 0; i < m->num_nodes * 3; ++i)
    if (!std::isfinite(m->coords[i])) return set_error(FIERRO_EINVAL, "non-finite coordinate at %lld", (long long)i);
  return FIERRO_OK;
}

int validate_bcs(const fierro_boundary* bcs, int64_t num_bcs) {
  if (num_bcs < 0 || (num_bcs > 0 && !bcs)) return set_error(FIERRO_EINVAL, "bad boundary list");
  for (int64_t s = 0; s < num_bcs; ++s) {
    if (bcs[s].surface < 0 || bcs[s].surface > 4)
      return set_error(FIERRO_EINVAL, "boundary %lld: surface tag %d unknown", (long long)s, bcs[s].surface);
    if (bcs[s].hydro_bc < 0 || bcs[s].hydro_bc > 5)
      return set_error(FIERRO_EINVAL, "boundary %lld: hydro_bc %d unknown (fixed 0, reflected 1, velocity 2, "
                       "pressure 3, acceleration 4, contact 5)", (long long)s, bcs[s].hydro_bc);
    if (bcs[s].hydro_bc == 1 && bcs[s].surface > 2)
      return set_error(FIERRO_EINVAL, "boundary %lld: a reflected condition needs a plane surface", (long long)s);
  }
  return FIERRO_OK;
}

int build_topology(const fierro_mesh* mesh, const fierro_boundary* bcs, int64_t num_bcs, bool renumber,
                   HostTopo* t) {
  int rc = validate_mesh(mesh);
  if (rc) return rc;
  rc = validate_bcs(bcs, num_bcs);
  if (rc) return rc;
  const int64_t nn = mesh->num_nodes, ne = mesh->num_elems;
  const uint64_t* nie = mesh->nodes_in_elem;
  t->nn = nn;
  t->ne = ne;
  // ---- renumbering
  if (renumber) {
    std::vector<double> cen((size_t)ne * 3);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < ne; ++e)
      for (int d = 0; d < 3; ++d) {
        double s = 0;
        for (int l = 0; l < 8; ++l) s += mesh->coords[nie[e * 8 + l] * 3 + d];
        cen[e * 3 + d] = s * 0.125;
      }
    t->elem_int2ext = radix_order(morton_keys(cen.data(), ne));
    t->node_int2ext = radix_order(morton_keys(mesh->coords, nn));
  } else {
    t->elem_int2ext.resize((size_t)ne);
    std::iota(t->elem_int2ext.begin(), t->elem_int2ext.end(), 0);
    t->node_int2ext.resize((size_t)nn);
    std::iota(t->node_int2ext.begin(), t->node_int2ext.end(), 0);
  }
  t->elem_ext2int.resize((size_t)ne);
  t->node_ext2int.resize((size_t)nn);
  for (int64_t i = 0; i < ne; ++i) t->elem_ext2int[t->elem_int2ext[i]] = i;
  for (int64_t i = 0; i < nn; ++i) t->node_ext2int[t->node_int2ext[i]] = i;
  // ---- element -> node in the internal numbering, local order kept
  t->nie.resize((size_t)ne * 8);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < ne; ++e) {
    int64_t E = t->elem_int2ext[e];
    for (int l = 0; l < 8; ++l) t->nie[e * 8 + l] = (int32_t)t->node_ext2int[nie[E * 8 + l]];
  }
  // ---- corner CSR per internal node, in ascending external element id
  t->cin_start.assign((size_t)nn + 1, 0);
  for (int64_t i = 0; i < ne * 8; ++i) t->cin_start[t->nie[i] + 1]++;
  for (int64_t n = 0; n < nn; ++n) t->cin_start[n + 1] += t->cin_start[n];
  t->max_corners_per_node = 0;
  for (int64_t n = 0; n < nn; ++n)
    t->max_corners_per_node = std::max(t->max_corners_per_node, t->cin_start[n + 1] - t->cin_start[n]);
  t->cin.resize((size_t)ne * 8);
  {
    std::vector<int32_t> fill(t->cin_start.begin(), t->cin_start.end() - 1);
    for (int64_t E = 0; E < ne; ++E) {
      int64_t e = t->elem_ext2int[E];
      for (int l = 0; l < 8; ++l) {
        int64_t n = t->node_ext2int[nie[E * 8 + l]];
        t->cin[fill[n]++] = (int32_t)(e * 8 + l);
      }
    }
  }
  // ---- neighbours: every other element sharing a node (mesh.h:274-322)
  std::vector<int32_t> cnt((size_t)ne);
  auto neighbours = [&](int64_t e, int32_t* out) -> int {
    int k = 0;
    for (int l = 0; l < 8; ++l) {
      int32_t n = t->nie[e * 8 + l];
      for (int32_t c = t->cin_start[n]; c < t->cin_start[n + 1]; ++c) {
        int32_t o = t->cin[c] >> 3;
        if (o == e) continue;
        bool seen = false;
        for (int i = 0; i < k; ++i)
          if (out[i] == o) { seen = true; break; }
        if (!seen && k < 256) out[k++] = o;
      }
    }
    return k;
  };
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < ne; ++e) {
    int32_t buf[256];
    cnt[e] = neighbours(e, buf);
  }
  t->eie_start.assign((size_t)ne + 1, 0);
  for (int64_t e = 0; e < ne; ++e) t->eie_start[e + 1] = t->eie_start[e] + cnt[e];
  t->eie.resize((size_t)t->eie_start[ne]);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < ne; ++e) neighbours(e, t->eie.data() + t->eie_start[e]);
  // ---- boundary masks
  std::vector<uint8_t> mask_ext;
  rc = boundary_masks(mesh, bcs, num_bcs, mesh->coords, &mask_ext, nullptr);
  if (rc) return rc;
  t->bc_mask.resize((size_t)nn);
  for (int64_t n = 0; n < nn; ++n) t->bc_mask[n] = mask_ext[t->node_int2ext[n]];
  return FIERRO_OK;
}

}  // namespace fierro

using namespace fierro;

extern "C" const char* fierro_last_error(void) { return fierro::g_err.c_str(); }
extern "C" const char* fierro_version(void) { return "fierro-sgh-gb300 0.1.0"; }

// setup (setup.cpp:10-424), after get_vol (driver.cpp:239), in the caller's numbering.
extern "C" int fierro_sgh_setup(const fierro_mesh* mesh, const fierro_material* materials,
                                int64_t num_materials, const double* state_vars, int64_t num_state_vars,
                                const fierro_mat_fill* fills, int64_t num_fills,
                                const fierro_boundary* boundaries, int64_t num_bcs, fierro_sgh_state* out) {
  clear_error();
  int rc = check_mesh_header(mesh);
  if (rc) return rc;
  if (mesh_dims(mesh) == 2)
    return rz::setup(mesh, materials, num_materials, state_vars, num_state_vars, fills, num_fills, boundaries,
                     num_bcs, out);
  rc = validate_bcs(boundaries, num_bcs);
  if (rc) return rc;
  if (!out || !out->node_coords || !out->node_vel || !out->node_mass || !out->elem_den || !out->elem_pres ||
      !out->elem_sspd || !out->elem_sie || !out->elem_vol || !out->elem_mass || !out->elem_mat_id ||
      !out->elem_statev)
    return set_error(FIERRO_EINVAL, "setup: output state arrays missing");
  if (num_materials < 1 || !materials || num_state_vars < 2 || !state_vars)
    return set_error(FIERRO_EINVAL, "setup: need >=1 material and >=2 state variables");
  if (out->num_state_vars != num_state_vars)
    return set_error(FIERRO_EINVAL, "setup: state.num_state_vars (%lld) != num_state_vars (%lld)",
                     (long long)out->num_state_vars, (long long)num_state_vars);
  for (int64_t m = 0; m < num_materials; ++m) {
    if (materials[m].eos_model != 0) return set_error(FIERRO_ENOTSUP, "material %lld: only the ideal-gas EOS", (long long)m);
    if (materials[m].strength_type < 0 || materials[m].strength_type > 2)
      return set_error(FIERRO_EINVAL, "material %lld: strength_type %d unknown (0 none, 1 hypo, 2 hyper)",
                       (long long)m, materials[m].strength_type);
  }
  for (int64_t f = 0; f < num_fills; ++f) {
    if (fills[f].mat_id < 0 || fills[f].mat_id >= num_materials)
      return set_error(FIERRO_EINVAL, "fill %lld: material id %d out of range", (long long)f, fills[f].mat_id);
    if (fills[f].volume < 0 || fills[f].volume > 3)
      return set_error(FIERRO_EINVAL, "fill %lld: region %d unknown", (long long)f, fills[f].volume);
    int v = fills[f].velocity;
    if (v != 0 && v != 1 && v != 2 && v != 3 && v != 4 && v != 5)
      return set_error(FIERRO_EINVAL, "fill %lld: velocity type %d unknown", (long long)f, v);
    if (v == 5 && num_state_vars < 5)
      return set_error(FIERRO_EINVAL, "fill %lld: tg_vortex reads statev(4)", (long long)f);
  }
  {
    const char* env = std::getenv("FIERRO_STAGED_TRANSFERS");
    if (!(env && env[0] == '1') && setup_gpu::usable(fills, num_fills))
      return setup_gpu::run(mesh, state_vars, num_state_vars, fills, num_fills, boundaries, num_bcs, out);
  }
  rc = validate_mesh(mesh);
  if (rc) return rc;
  const int64_t nn = mesh->num_nodes, ne = mesh->num_elems, nsv = num_state_vars;
  const uint64_t* nie = mesh->nodes_in_elem;
  double* X = out->node_coords;
  double* V = out->node_vel;
  double* X1 = X + nn * 3;
  double* V1 = V + nn * 3;
  // read_mesh_ensight leaves the coordinates in both bins (read_mesh.cpp:129-137)
  std::memcpy(X, mesh->coords, sizeof(double) * (size_t)nn * 3);
  std::memcpy(X1, mesh->coords, sizeof(double) * (size_t)nn * 3);
  std::memset(V, 0, sizeof(double) * (size_t)nn * 6);
  std::memset(out->node_mass, 0, sizeof(double) * (size_t)nn);
  std::memset(out->elem_den, 0, sizeof(double) * (size_t)ne);
  std::memset(out->elem_pres, 0, sizeof(double) * (size_t)ne);
  std::memset(out->elem_sspd, 0, sizeof(double) * (size_t)ne);
  std::memset(out->elem_sie, 0, sizeof(double) * (size_t)ne * 2);
  std::memset(out->elem_mass, 0, sizeof(double) * (size_t)ne);
  std::memset(out->elem_mat_id, 0, sizeof(uint64_t) * (size_t)ne);
  std::memset(out->elem_statev, 0, sizeof(double) * (size_t)(ne * nsv));
  if (out->elem_stress) std::memset(out->elem_stress, 0, sizeof(double) * (size_t)ne * 18);
  if (out->elem_div) std::memset(out->elem_div, 0, sizeof(double) * (size_t)ne);
  if (out->corner_force) std::memset(out->corner_force, 0, sizeof(double) * (size_t)ne * 24);
  double* vol = out->elem_vol;
  // get_vol (geometry.cpp:238-267)
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < ne; ++e) {
    double x[8], y[8], z[8];
    for (int l = 0; l < 8; ++l) {
      const double* c = X1 + nie[e * 8 + l] * 3;
      x[l] = c[0];
      y[l] = c[1];
      z[l] = c[2];
    }
    vol[e] = hex::volume(x, y, z);
  }
  // an inverted or degenerate element makes every later density and force
  // meaningless; the reference does not check, this library refuses the mesh
  for (int64_t e = 0; e < ne; ++e)
    if (!(vol[e] > 0.0) || !std::isfinite(vol[e]))
      return set_error(FIERRO_ENUMERIC, "setup: element %lld has volume %g (inverted or degenerate)",
                       (long long)e, vol[e]);
  // boundary node sets (setup.cpp:37-43)
  std::vector<uint8_t> mask;
  rc = boundary_masks(mesh, boundaries, num_bcs, X1, &mask, nullptr);
  if (rc) return rc;
  const double PI = 3.141592653589793;
  // fills (setup.cpp:109-357)
  for (int64_t fi = 0; fi < num_fills; ++fi) {
    const fierro_mat_fill& F = fills[fi];
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < ne; ++e) {
      double ec[3] = {0.0, 0.0, 0.0};
      for (int l = 0; l < 8; ++l) {
        const double* c = X1 + nie[e * 8 + l] * 3;
        ec[0] += c[0];
        ec[1] += c[1];
        ec[2] += c[2];
      }
      ec[0] = ec[0] / 8;
      ec[1] = ec[1] / 8;
      ec[2] = ec[2] / 8;
      double radius = std::sqrt(ec[0] * ec[0] + ec[1] * ec[1] + ec[2] * ec[2]);
      double radius_cyl = std::sqrt(ec[0] * ec[0] + ec[1] * ec[1]);
      bool fill_this = false;
      switch (F.volume) {
        case 0: fill_this = true; break;
        case 1:
          fill_this = ec[0] >= F.x1 && ec[0] <= F.x2 && ec[1] >= F.y1 && ec[1] <= F.y2 && ec[2] >= F.z1 &&
                      ec[2] <= F.z2;
          break;
        case 2: fill_this = radius_cyl >= F.radius1 && radius_cyl <= F.radius2; break;
        case 3: fill_this = radius >= F.radius1 && radius <= F.radius2; break;
      }
      if (!fill_this) continue;
      double* sv = out->elem_statev + e * nsv;
      out->elem_den[e] = F.den;
      out->elem_mass[e] = out->elem_den[e] * vol[e];
      out->elem_sie[ne + e] = F.sie;
      out->elem_mat_id[e] = (uint64_t)F.mat_id;
      for (int64_t v = 0; v < nsv; ++v) sv[v] = state_vars[F.mat_id * nsv + v];
      if (out->elem_stress)
        for (int k = 0; k < 9; ++k) out->elem_stress[ne * 9 + e * 9 + k] = 0.0;
      // ideal_gas (eos.cpp:12-46)
      double gamma = sv[0], csmin = sv[1];
      out->elem_pres[e] = (gamma - 1.0) * out->elem_sie[ne + e] * out->elem_den[e];
      out->elem_sspd[e] = std::sqrt(gamma * (gamma - 1.0) * out->elem_sie[ne + e]);
      if (out->elem_sspd[e] < csmin) out->elem_sspd[e] = csmin;
      for (int l = 0; l < 8; ++l) {
        const uint64_t n = nie[e * 8 + l];
        const double* c = X1 + n * 3;
        double* v = V1 + n * 3;
        if (F.velocity == 0) {
          v[0] = F.u;
          v[1] = F.v;
          v[2] = F.w;
        } else if (F.velocity == 1 || F.velocity == 2) {
          const int nd = (F.velocity == 1) ? 2 : 3;
          double dir[3] = {0.0, 0.0, 0.0};
          double radius_val = 0.0;
          for (int d = 0; d < nd; ++d) {
            dir[d] = c[d];
            radius_val += c[d] * c[d];
          }
          radius_val = std::sqrt(radius_val);
          for (int d = 0; d < nd; ++d) {
            if (radius_val > 1.0e-14) dir[d] /= (radius_val);
            else dir[d] = 0.0;
          }
          v[0] = F.speed * dir[0];
          v[1] = F.speed * dir[1];
          v[2] = (nd == 3) ? F.speed * dir[2] : 0.0;
        } else if (F.velocity == 5) {
          v[0] = std::sin(PI * c[0]) * std::cos(PI * c[1]);
          v[1] = -1.0 * std::cos(PI * c[0]) * std::sin(PI * c[1]);
          v[2] = 0.0;
        }
      }
      if (F.velocity == 5) {
        out->elem_pres[e] = 0.25 * (std::cos(2.0 * PI * ec[0]) + std::cos(2.0 * PI * ec[1])) + 1.0;
        double g4 = sv[4];
        out->elem_sie[ne + e] = out->elem_pres[e] / (F.den * (g4 - 1.0));
      }
    }
  }
  // boundary_velocity (setup.cpp:362)
  for (int64_t n = 0; n < nn; ++n)
    for (int d = 0; d < 3; ++d)
      if (mask[n] & (1u << d)) V1[n * 3 + d] = 0.0;
  // node mass, sum over elems_in_node in corner order (setup.cpp:394-420)
  std::vector<int64_t> start, elems;
  node_elem_csr(nn, ne, nie, &start, &elems, nullptr);
#pragma omp parallel for schedule(static)
  for (int64_t n = 0; n < nn; ++n) {
    double m = 0.0;
    for (int64_t k = start[n]; k < start[n + 1]; ++k) m += 1.0 / 8.0 * out->elem_mass[elems[k]];
    out->node_mass[n] = m;
  }
  return FIERRO_OK;
}
