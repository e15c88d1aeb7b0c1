// 2D-RZ (num_dims == 2) host side: quad-mesh validation and topology (Morton
// renumbering, corner and neighbour CSRs, boundary edges and masks, the
// boundary nodes with their edge neighbours for the axis mass fix), the handle's
// device arrays, state transfers through the pinned staging buffers, the stage
// launches, the energy tallies, and setup (setup.cpp:10-424) for quad meshes.
// Compiled with -ffp-contract=off so the set-up doubles are uncontracted.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#include "sgh_handle.h"
#include "sgh_rz.h"
#include "sgh_user_mat.cuh"
#include "sgh_xfer.h"

namespace fierro {

namespace {

// Quad edges as patches (mesh.h:364-373); the edge neighbours of local node l
// are (l+1)&3 and (l+3)&3.
constexpr int kEdge[4][2] = {{0, 3}, {1, 2}, {0, 1}, {3, 2}};

int validate_mesh_rz(const fierro_mesh* m) {
  int rc = check_mesh_header(m);
  if (rc) return rc;
  for (int64_t e = 0; e < m->num_elems; ++e)
    for (int l = 0; l < 4; ++l) {
      const uint64_t n = m->nodes_in_elem[e * 4 + l];
      if (n >= (uint64_t)m->num_nodes)
        return set_error(FIERRO_EINVAL, "element %lld node %d id %llu out of range", (long long)e, l,
                         (unsigned long long)n);
      for (int k = 0; k < l; ++k)
        if (m->nodes_in_elem[e * 4 + k] == n)
          return set_error(FIERRO_EINVAL, "element %lld repeats node %llu", (long long)e, (unsigned long long)n);
    }
  for (int64_t i = 0; i < m->num_nodes * 2; ++i)
    if (!std::isfinite(m->coords[i])) return set_error(FIERRO_EINVAL, "non-finite coordinate at %lld", (long long)i);
  return FIERRO_OK;
}

// Node -> (element, local node) CSR in the caller's numbering, elements ascending
// per node: the corner order of build_corner_connectivity (mesh.h:218-241).
void node_corner_csr(int64_t nn, int64_t ne, const uint64_t* nie, std::vector<int64_t>* start,
                     std::vector<int64_t>* corners) {
  start->assign((size_t)nn + 1, 0);
  for (int64_t i = 0; i < ne * 4; ++i) (*start)[nie[i] + 1]++;
  for (int64_t n = 0; n < nn; ++n) (*start)[n + 1] += (*start)[n];
  corners->resize((size_t)ne * 4);
  std::vector<int64_t> fill(start->begin(), start->end() - 1);
  for (int64_t e = 0; e < ne; ++e)
    for (int l = 0; l < 4; ++l) (*corners)[fill[nie[e * 4 + l]]++] = e * 4 + l;
}

bool elem_has_node(const uint64_t* nie, int64_t e, uint64_t n) {
  for (int l = 0; l < 4; ++l)
    if (nie[e * 4 + l] == n) return true;
  return false;
}

// check_bdy (setup.cpp:487-571) for one node of an edge, 2D: x plane, y plane,
// cylinder sqrt(x^2 + y^2).
bool on_surface(const double* c, int tag, double val) {
  if (tag == 0) return std::fabs(c[0] - val) <= 1.0e-7;
  if (tag == 1) return std::fabs(c[1] - val) <= 1.0e-7;
  if (tag == 3) return std::fabs(std::sqrt(c[0] * c[0] + c[1] * c[1]) - val) <= 1.0e-7;
  return false;
}

// Boundary edges (mesh.h:342-570: an edge no other element has), the
// boundary-condition mask per external node (setup.cpp:431-665) and the set of
// boundary nodes (mesh.h:592-645).
void boundary_rz(const fierro_mesh* mesh, const fierro_boundary* bcs, int64_t num_bcs, const double* coords,
                 const std::vector<int64_t>& start, const std::vector<int64_t>& corners,
                 std::vector<uint8_t>* mask, std::vector<char>* on_bdy) {
  const int64_t nn = mesh->num_nodes, ne = mesh->num_elems;
  const uint64_t* nie = mesh->nodes_in_elem;
  std::vector<char> bdy_edge((size_t)ne * 4, 0);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < ne; ++e)
    for (int p = 0; p < 4; ++p) {
      const uint64_t a = nie[e * 4 + kEdge[p][0]], b = nie[e * 4 + kEdge[p][1]];
      bool shared = false;
      for (int64_t k = start[a]; k < start[a + 1] && !shared; ++k) {
        const int64_t o = corners[k] / 4;
        if (o != e && elem_has_node(nie, o, b)) shared = true;
      }
      bdy_edge[e * 4 + p] = !shared;
    }
  std::vector<int64_t> edges;  // e*4 + p of the boundary edges
  for (int64_t i = 0; i < ne * 4; ++i)
    if (bdy_edge[i]) edges.push_back(i);
  mask->assign((size_t)nn, 0);
  on_bdy->assign((size_t)nn, 0);
  for (int64_t pe : edges) {
    const int64_t e = pe / 4;
    const int p = (int)(pe % 4);
    (*on_bdy)[nie[e * 4 + kEdge[p][0]]] = 1;
    (*on_bdy)[nie[e * 4 + kEdge[p][1]]] = 1;
  }
  for (int64_t s = 0; s < num_bcs; ++s) {
    // reflected: the surface's component (x plane -> u, y plane -> v); fixed: both
    const uint8_t bits = bc_mask_bits(bcs[s].hydro_bc, bcs[s].surface, 2);
    for (int64_t pe : edges) {
      const int64_t e = pe / 4;
      const int p = (int)(pe % 4);
      const uint64_t a = nie[e * 4 + kEdge[p][0]], b = nie[e * 4 + kEdge[p][1]];
      if (on_surface(coords + a * 2, bcs[s].surface, bcs[s].value) &&
          on_surface(coords + b * 2, bcs[s].surface, bcs[s].value)) {
        (*mask)[a] |= bits;
        (*mask)[b] |= bits;
      }
    }
  }
}

double vol_quad(const double x[4], const double y[4]) {
  return ((y[2] + y[3] + y[0]) * ((y[2] - y[3]) * (x[0] - x[3]) - (y[0] - y[3]) * (x[2] - x[3])) +
          (y[0] + y[1] + y[2]) * ((y[0] - y[1]) * (x[2] - x[1]) - (y[2] - y[1]) * (x[0] - x[1]))) /
         6.0;
}

double heron(double x1, double y1, double x2, double y2, double x3, double y3) {
  double S = 0.0;
  const double a = std::sqrt((x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1));
  S += a;
  const double b = std::sqrt((x3 - x2) * (x3 - x2) + (y3 - y2) * (y3 - y2));
  S += b;
  const double c = std::sqrt((x3 - x1) * (x3 - x1) + (y3 - y1) * (y3 - y1));
  S += c;
  S *= 0.5;
  return std::sqrt(S * (S - a) * (S - b) * (S - c));
}

// get_area_weights2D (geometry.cpp:503-547)
void corner_areas(const double x[4], const double y[4], double ca[4]) {
  double rc = 0.0, zc = 0.0;
  for (int l = 0; l < 4; ++l) {
    rc += 0.25 * y[l];
    zc += 0.25 * x[l];
  }
  const double A12 = heron(x[0], y[0], zc, rc, x[1], y[1]);
  const double A23 = heron(x[1], y[1], zc, rc, x[2], y[2]);
  const double A34 = heron(x[2], y[2], zc, rc, x[3], y[3]);
  const double A41 = heron(x[3], y[3], zc, rc, x[0], y[0]);
  ca[0] = (5. * A41 + 5. * A12 + A23 + A34) / 12.;
  ca[1] = (A41 + 5. * A12 + 5. * A23 + A34) / 12.;
  ca[2] = (A41 + A12 + 5. * A23 + 5. * A34) / 12.;
  ca[3] = (5. * A41 + A12 + A23 + 5. * A34) / 12.;
}

}  // namespace

int validate_bcs_rz(const fierro_boundary* bcs, int64_t num_bcs) {
  if (num_bcs < 0 || (num_bcs > 0 && !bcs)) return set_error(FIERRO_EINVAL, "bad boundary list");
  for (int64_t s = 0; s < num_bcs; ++s) {
    const int t = bcs[s].surface;
    if (t != 0 && t != 1 && t != 3)
      return set_error(FIERRO_EINVAL, "boundary %lld: surface %d on a 2D-RZ mesh (x plane 0, y plane 1, "
                       "cylinder 3)", (long long)s, t);
    if (bcs[s].hydro_bc < 0 || bcs[s].hydro_bc > 5)
      return set_error(FIERRO_EINVAL, "boundary %lld: hydro_bc %d unknown (fixed 0, reflected 1, velocity 2, "
                       "pressure 3, acceleration 4, contact 5)", (long long)s, bcs[s].hydro_bc);
    if (bcs[s].hydro_bc == 1 && t == 3)
      return set_error(FIERRO_EINVAL, "boundary %lld: a reflected condition needs a plane surface", (long long)s);
  }
  return FIERRO_OK;
}

int build_topology_rz(const fierro_mesh* mesh, const fierro_boundary* bcs, int64_t num_bcs, HostTopo* t) {
  int rc = validate_mesh_rz(mesh);
  if (rc) return rc;
  rc = validate_bcs_rz(bcs, num_bcs);
  if (rc) return rc;
  const int64_t nn = mesh->num_nodes, ne = mesh->num_elems;
  const uint64_t* nie = mesh->nodes_in_elem;
  t->nn = nn;
  t->ne = ne;
  t->npe = 4;
  // ---- Morton renumbering of element centroids and nodes (z = 0)
  {
    std::vector<double> pts((size_t)std::max(nn, ne) * 3, 0.0);
    for (int64_t e = 0; e < ne; ++e)
      for (int d = 0; d < 2; ++d) {
        double s = 0;
        for (int l = 0; l < 4; ++l) s += mesh->coords[nie[e * 4 + l] * 2 + d];
        pts[e * 3 + d] = s * 0.25;
      }
    t->elem_int2ext = morton_order(pts.data(), ne);
    std::fill(pts.begin(), pts.end(), 0.0);
    for (int64_t n = 0; n < nn; ++n)
      for (int d = 0; d < 2; ++d) pts[n * 3 + d] = mesh->coords[n * 2 + d];
    t->node_int2ext = morton_order(pts.data(), nn);
  }
  t->elem_ext2int.resize((size_t)ne);
  t->node_ext2int.resize((size_t)nn);
  for (int64_t i = 0; i < ne; ++i) t->elem_ext2int[t->elem_int2ext[i]] = i;
  for (int64_t i = 0; i < nn; ++i) t->node_ext2int[t->node_int2ext[i]] = i;
  t->nie.resize((size_t)ne * 4);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < ne; ++e)
    for (int l = 0; l < 4; ++l) t->nie[e * 4 + l] = (int32_t)t->node_ext2int[nie[t->elem_int2ext[e] * 4 + l]];
  // ---- corner CSR per internal node, in ascending external element id
  std::vector<int64_t> start, corners;
  node_corner_csr(nn, ne, nie, &start, &corners);
  t->cin_start.assign((size_t)nn + 1, 0);
  t->cin.resize((size_t)ne * 4);
  t->max_corners_per_node = 0;
  for (int64_t i = 0; i < nn; ++i) {
    const int64_t n = t->node_int2ext[i];
    const int64_t cnt = start[n + 1] - start[n];
    t->cin_start[i + 1] = t->cin_start[i] + (int32_t)cnt;
    t->max_corners_per_node = std::max<int>(t->max_corners_per_node, (int)cnt);
    for (int64_t k = 0; k < cnt; ++k) {
      const int64_t c = corners[start[n] + k];
      t->cin[t->cin_start[i] + k] = (int32_t)(t->elem_ext2int[c / 4] * 4 + c % 4);
    }
  }
  // ---- neighbours: every other element sharing a node (mesh.h:249-338)
  auto neighbours = [&](int64_t e, int32_t* out) -> int {
    int k = 0;
    for (int l = 0; l < 4; ++l) {
      const int32_t n = t->nie[e * 4 + l];
      for (int32_t c = t->cin_start[n]; c < t->cin_start[n + 1]; ++c) {
        const int32_t o = t->cin[c] >> 2;
        if (o == e) continue;
        bool seen = false;
        for (int i = 0; i < k; ++i)
          if (out[i] == o) seen = true;
        if (!seen && k < 64) out[k++] = o;
      }
    }
    return k;
  };
  std::vector<int32_t> cnt((size_t)ne);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < ne; ++e) {
    int32_t buf[64];
    cnt[e] = neighbours(e, buf);
  }
  t->eie_start.assign((size_t)ne + 1, 0);
  for (int64_t e = 0; e < ne; ++e) t->eie_start[e + 1] = t->eie_start[e] + cnt[e];
  t->eie.resize((size_t)t->eie_start[ne]);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < ne; ++e) neighbours(e, t->eie.data() + t->eie_start[e]);
  // ---- boundary masks, boundary nodes and their edge neighbours
  std::vector<uint8_t> mask;
  std::vector<char> on_bdy;
  boundary_rz(mesh, bcs, num_bcs, mesh->coords, start, corners, &mask, &on_bdy);
  t->bc_mask.resize((size_t)nn);
  for (int64_t i = 0; i < nn; ++i) t->bc_mask[i] = mask[t->node_int2ext[i]];
  t->axis_nodes.clear();
  t->axis_nin_start.assign(1, 0);
  t->axis_nin.clear();
  for (int64_t i = 0; i < nn; ++i) {
    const int64_t n = t->node_int2ext[i];
    if (!on_bdy[n]) continue;
    t->axis_nodes.push_back((int32_t)i);
    std::vector<int32_t> nb;
    for (int64_t k = start[n]; k < start[n + 1]; ++k) {
      const int64_t c = corners[k], e = c / 4;
      const int l = (int)(c % 4);
      for (int m : {(l + 1) & 3, (l + 3) & 3}) {
        const int32_t j = (int32_t)t->node_ext2int[nie[e * 4 + m]];
        if (std::find(nb.begin(), nb.end(), j) == nb.end()) nb.push_back(j);
      }
    }
    t->axis_nin.insert(t->axis_nin.end(), nb.begin(), nb.end());
    t->axis_nin_start.push_back((int32_t)t->axis_nin.size());
  }
  return FIERRO_OK;
}

namespace rz {

using namespace hd;

int create(fierro_sgh* h, const fierro_mesh* mesh, const fierro_material* materials, int64_t num_materials,
           const fierro_boundary* boundaries, int64_t num_bcs) {
  if (h->has_hyper)
    return set_error(FIERRO_ENOTSUP, "hyper strength models on a 2D-RZ mesh: the reference's update_state2D "
                     "(properties.cpp:146-160) writes 3D corner normals into a 2D array");
  TRY(build_topology_rz(mesh, boundaries, num_bcs, &h->topo));
  {
    // set/get_state through the transfer kernels (sgh_xfer.cu) where the GPU
    // dereferences host memory, staged through pinned buffers otherwise
    const char* env = std::getenv("FIERRO_STAGED_TRANSFERS");
    h->direct_host = xfer::direct_host_access() && !(env && env[0] == '1');
  }
  h->rks = (h->fp_mode == FIERRO_FP_EXACT) ? &rz_kernels_exact() : &rz_kernels_fma();
  const size_t nn = (size_t)h->nn, ne = (size_t)h->ne;
  const HostTopo& t = h->topo;
  TRY(dalloc(h, &h->d_nie, ne * 4));
  TRY(dalloc(h, &h->d_cin_start, nn + 1));
  TRY(dalloc(h, &h->d_cin, ne * 4));
  TRY(dalloc(h, &h->d_eie_start, ne + 1));
  TRY(dalloc(h, &h->d_eie, t.eie.size()));
  TRY(dalloc(h, &h->d_mat, ne));
  TRY(dalloc(h, &h->d_bc, nn));
  TRY(dalloc(h, &h->d_qtab, (size_t)num_materials * 4));
  TRY(dalloc(h, &h->d_node_mass, nn));
  TRY(dalloc(h, &h->d_node_ext, nn));
  TRY(dalloc(h, &h->d_rad, nn));
  TRY(dalloc(h, &h->d_elem_mass, ne));
  TRY(dalloc(h, &h->d_gamma, ne));
  TRY(dalloc(h, &h->d_csmin, ne));
  for (int b = 0; b < 2; ++b)
    for (int d = 0; d < 2; ++d) {
      TRY(dalloc(h, &h->d_x[b][d], nn));
      TRY(dalloc(h, &h->d_v[b][d], nn));
    }
  for (int d = 0; d < 2; ++d) TRY(dalloc(h, &h->d_h[d], nn));
  TRY(dalloc(h, &h->d_den, ne));
  TRY(dalloc(h, &h->d_pres, ne));
  TRY(dalloc(h, &h->d_sspd, ne));
  TRY(dalloc(h, &h->d_vol, ne));
  TRY(dalloc(h, &h->d_div[0], ne));
  TRY(dalloc(h, &h->d_div[1], ne));
  TRY(dalloc(h, &h->d_sie[0], ne));
  TRY(dalloc(h, &h->d_sie[1], ne));
  TRY(dalloc(h, &h->d_force, ne * 8));
  if (h->strength) {
    TRY(dalloc(h, &h->d_stress[0], ne * 9));
    TRY(dalloc(h, &h->d_stress[1], ne * 9));
    TRY(dalloc(h, &h->d_stype, (size_t)num_materials));
    std::vector<int> st((size_t)num_materials);
    for (int64_t m = 0; m < num_materials; ++m) st[m] = materials[m].strength_type;
    TRY(upload_raw(h, h->d_stype, st.data(), sizeof(int) * st.size()));
  }
  h->naxis = (int)t.axis_nodes.size();
  TRY(dalloc(h, &h->d_elem_int2ext, ne));
  {
    std::vector<int32_t> m32(ne);
    for (size_t j = 0; j < ne; ++j) m32[j] = (int32_t)t.elem_int2ext[j];
    TRY(upload_raw(h, h->d_elem_int2ext, m32.data(), sizeof(int32_t) * ne));
  }
  if (h->direct_host) {
    // caller -> internal maps and the validation word of the transfer kernels
    TRY(dalloc(h, &h->d_node_ext2int, nn));
    TRY(dalloc(h, &h->d_elem_ext2int, ne));
    TRY(dalloc(h, &h->d_xfer, 1));
    std::vector<int32_t> m32(std::max(nn, ne));
    for (size_t j = 0; j < nn; ++j) m32[j] = (int32_t)t.node_ext2int[j];
    TRY(upload_raw(h, h->d_node_ext2int, m32.data(), sizeof(int32_t) * nn));
    for (size_t j = 0; j < ne; ++j) m32[j] = (int32_t)t.elem_ext2int[j];
    TRY(upload_raw(h, h->d_elem_ext2int, m32.data(), sizeof(int32_t) * ne));
  }
  TRY(dalloc(h, &h->d_axis, t.axis_nodes.size()));
  TRY(dalloc(h, &h->d_axis_nin_start, t.axis_nin_start.size()));
  TRY(dalloc(h, &h->d_axis_nin, t.axis_nin.size()));
  h->ncfl = (int)((ne + kElemBlock - 1) / kElemBlock);
  TRY(dalloc(h, &h->d_cfl, (size_t)h->ncfl));
  TRY(dalloc(h, &h->d_ctrl, 1));
  TRY(dalloc(h, &h->d_energy_part, 2 * 512));
  TRY(dalloc(h, &h->d_energy_out, 2));
  h->stage_elems = std::max(nn, ne);
  for (int i = 0; i < 2; ++i) {
    CUDA_TRY(cudaHostAlloc((void**)&h->h_stage[i], sizeof(double) * h->stage_elems, cudaHostAllocDefault));
    CUDA_TRY(cudaEventCreateWithFlags(&h->stage_ev[i], cudaEventDisableTiming));
    CUDA_TRY(cudaEventRecord(h->stage_ev[i], h->stream));
  }
  TRY(upload_raw(h, h->d_nie, t.nie.data(), sizeof(int32_t) * ne * 4));
  TRY(upload_raw(h, h->d_cin_start, t.cin_start.data(), sizeof(int32_t) * (nn + 1)));
  TRY(upload_raw(h, h->d_cin, t.cin.data(), sizeof(int32_t) * ne * 4));
  TRY(upload_raw(h, h->d_eie_start, t.eie_start.data(), sizeof(int32_t) * (ne + 1)));
  if (!t.eie.empty()) TRY(upload_raw(h, h->d_eie, t.eie.data(), sizeof(int32_t) * t.eie.size()));
  TRY(upload_raw(h, h->d_bc, t.bc_mask.data(), nn));
  if (!t.axis_nodes.empty()) TRY(upload_raw(h, h->d_axis, t.axis_nodes.data(), sizeof(int32_t) * t.axis_nodes.size()));
  TRY(upload_raw(h, h->d_axis_nin_start, t.axis_nin_start.data(), sizeof(int32_t) * t.axis_nin_start.size()));
  if (!t.axis_nin.empty()) TRY(upload_raw(h, h->d_axis_nin, t.axis_nin.data(), sizeof(int32_t) * t.axis_nin.size()));
  h->nnz_eie = (int64_t)t.eie.size();
  std::vector<double> q((size_t)num_materials * 4);
  for (int64_t m = 0; m < num_materials; ++m) {
    q[m * 4 + 0] = materials[m].q1;
    q[m * 4 + 1] = materials[m].q1ex;
    q[m * 4 + 2] = materials[m].q2;
    q[m * 4 + 3] = materials[m].q2ex;
  }
  TRY(upload_raw(h, h->d_qtab, q.data(), sizeof(double) * q.size()));
  CUDA_TRY(cudaMemsetAsync(h->d_ctrl, 0, sizeof(Ctrl), h->stream));
  CUDA_TRY(cudaMemsetAsync(h->d_force, 0, sizeof(double) * ne * 8, h->stream));
  return FIERRO_OK;
}

int set_state(fierro_sgh* h, const fierro_sgh_state* s) {
  const int64_t nn = h->nn, ne = h->ne, nsv = s->num_state_vars;
  const HostTopo& t = h->topo;
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
  int slot = 0;
  // reference bin 1 -> device bin 0 (current), bin 0 -> device bin 1
  for (int rb = 0; rb < 2; ++rb) {
    const int b = rb ^ 1;
    for (int d = 0; d < 2; ++d) {
      TRY(upload_gather(h, h->d_x[b][d], s->node_coords + (size_t)rb * nn * 2, t.node_int2ext, 2, d, &slot));
      TRY(upload_gather(h, h->d_v[b][d], s->node_vel + (size_t)rb * nn * 2, t.node_int2ext, 2, d, &slot));
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
  if (s->elem_div) TRY(upload_gather(h, h->d_div[1], s->elem_div, t.elem_int2ext, 1, 0, &slot));
  else CUDA_TRY(cudaMemsetAsync(h->d_div[1], 0, sizeof(double) * (size_t)ne, h->stream));
  return FIERRO_OK;
}

static RzElemArgs elem_args_rz(fierro_sgh* h, int cur, int c, double alpha, int div_out) {
  RzElemArgs a{};
  a.ne = (int)h->ne;
  a.nie = h->d_nie;
  a.x = h->d_x[cur][0];
  a.y = h->d_x[cur][1];
  a.u = h->d_v[cur][0];
  a.v = h->d_v[cur][1];
  a.hx = h->d_h[0];
  a.hy = h->d_h[1];
  a.rad = h->d_rad;
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
  a.cfl_part = h->d_cfl;
  a.ctrl = h->d_ctrl;
  a.rk_alpha = alpha;
  a.dt_cfl = h->lp.dt_cfl;
  a.fuzz = h->lp.fuzz;
  return a;
}

// The uploaded state's divergence and CFL partials, and the extensive node mass
// m*y of the run that starts here (sgh_solve.cpp:106-114).
int prime(fierro_sgh* h) {
  h->rks->elem(elem_args_rz(h, 0, 0, 1.0, 0), 2, h->stream);
  h->rks->ext_mass((int)h->nn, h->d_node_mass, h->d_x[0][1], h->d_node_ext, h->stream);
  CUDA_TRY(cudaGetLastError());
  return FIERRO_OK;
}

int get_state(fierro_sgh* h, fierro_sgh_state* s, const int bins[2], int qb) {
  const int64_t nn = h->nn, ne = h->ne;
  const HostTopo& t = h->topo;
  for (int rb = 0; rb < 2; ++rb)
    for (int d = 0; d < 2; ++d) {
      if (s->node_coords)
        TRY(download_scatter(h, s->node_coords + (size_t)rb * nn * 2, h->d_x[bins[rb]][d], t.node_int2ext, 2, d));
      if (s->node_vel)
        TRY(download_scatter(h, s->node_vel + (size_t)rb * nn * 2, h->d_v[bins[rb]][d], t.node_int2ext, 2, d));
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
  if (s->corner_force)
    // device [lid*2+dim][e] -> reference [(E*4+lid)*2+dim]
    for (int r = 0; r < 8; ++r)
      TRY(download_scatter(h, s->corner_force, h->d_force + (size_t)r * ne, t.elem_int2ext, 8, (size_t)r));
  return FIERRO_OK;
}

int enqueue_stage(fierro_sgh* h, int c, int s, cudaEvent_t* ev, size_t* k) {
  const double alpha = stage_alpha(h, s);
  const int rb = (s == 0) ? c : (c ^ 1);
  const int q = div_parity(h, c, s);
  RzForceArgs f{};
  f.ne = (int)h->ne;
  f.nie = h->d_nie;
  f.eie_start = h->d_eie_start;
  f.eie = h->d_eie;
  f.mat = h->d_mat;
  f.qtab = h->d_qtab;
  f.x = h->d_x[rb][0];
  f.y = h->d_x[rb][1];
  f.u = h->d_v[rb][0];
  f.v = h->d_v[rb][1];
  f.den = h->d_den;
  f.pres = h->d_pres;
  f.sspd = h->d_sspd;
  f.vol = h->d_vol;
  f.div = h->d_div[q];
  f.force = h->d_force;
  f.ctrl = h->d_ctrl;
  f.fuzz = h->lp.fuzz;
  f.small = h->lp.small;
  if (h->strength) {
    f.stress_cur = h->d_stress[rb];
    f.stress0 = h->d_stress[c];
    f.stress_out = h->d_stress[c ^ 1];
    f.stype = h->d_stype;
    f.statev = h->d_statev;
    f.sie0 = h->d_sie[c];
    f.rk_alpha = alpha;
    f.copy_stress = s == 0;
  }
  RzNodeArgs n{};
  n.nn = (int)h->nn;
  n.ne = (int)h->ne;
  n.cin_start = h->d_cin_start;
  n.cin = h->d_cin;
  n.force = h->d_force;
  n.node_mass = h->d_node_mass;
  n.node_ext = h->d_node_ext;
  n.bc_mask = h->d_bc;
  n.u0 = h->d_v[c][0];
  n.v0 = h->d_v[c][1];
  n.x0 = h->d_x[c][0];
  n.y0 = h->d_x[c][1];
  n.u1 = h->d_v[c ^ 1][0];
  n.v1 = h->d_v[c ^ 1][1];
  n.x1 = h->d_x[c ^ 1][0];
  n.y1 = h->d_x[c ^ 1][1];
  n.yin = h->d_x[rb][1];
  n.hx = h->d_h[0];
  n.hy = h->d_h[1];
  n.rad = h->d_rad;
  n.ctrl = h->d_ctrl;
  n.rk_alpha = alpha;
  n.tiny = h->tiny;
  RzAxisArgs x{};
  x.naxis = h->naxis;
  x.nodes = h->d_axis;
  x.nin_start = h->d_axis_nin_start;
  x.nin = h->d_axis_nin;
  x.y1 = h->d_x[c ^ 1][1];
  x.node_mass = h->d_node_mass;
  x.ctrl = h->d_ctrl;
  x.tiny = h->tiny;
  const RzElemArgs e = elem_args_rz(h, c ^ 1, c, alpha, q ^ 1);
  auto mark = [&]() -> int {
    if (ev) CUDA_TRY(cudaEventRecord(ev[(*k)++], h->stream));
    return FIERRO_OK;
  };
  h->rks->force(f, h->stream);
  TRY(mark());
  h->rks->node(n, h->stream);
  TRY(mark());
  h->rks->axis(x, h->stream);
  TRY(mark());
  h->rks->elem(e, (s == h->rk_num_stages - 1) ? 1 : 0, h->stream);
  TRY(mark());
  return FIERRO_OK;
}

int energy(fierro_sgh* h, int bin, double* ie, double* ke) {
  RzEnergyArgs a{};
  a.ne = (int)h->ne;
  a.nn = (int)h->nn;
  a.mass = h->d_elem_mass;
  a.sie = h->d_sie[bin];
  a.node_mass = h->d_node_mass;
  a.u = h->d_v[bin][0];
  a.v = h->d_v[bin][1];
  a.y = h->d_x[bin][1];
  a.part = h->d_energy_part;
  a.out = h->d_energy_out;
  h->rks->energy(a, h->stream);
  double out[2];
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(out, h->d_energy_out, sizeof(out), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (ie) *ie = out[0];
  if (ke) *ke = out[1];
  return FIERRO_OK;
}

// setup (setup.cpp:10-424) with num_dims == 2, after get_vol (driver.cpp:239).
int setup(const fierro_mesh* mesh, const fierro_material* materials, int64_t num_materials,
          const double* state_vars, int64_t num_state_vars, const fierro_mat_fill* fills, int64_t num_fills,
          const fierro_boundary* boundaries, int64_t num_bcs, fierro_sgh_state* out) {
  int rc = validate_bcs_rz(boundaries, num_bcs);
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
    const int v = fills[f].velocity;
    if (v < 0 || v > 5) return set_error(FIERRO_EINVAL, "fill %lld: velocity type %d unknown", (long long)f, v);
    if (v == 2)
      return set_error(FIERRO_ENOTSUP, "fill %lld: the spherical velocity on a 2D-RZ mesh reads a third "
                       "coordinate (setup.cpp:272-296); use radial", (long long)f);
    if (v == 5 && num_state_vars < 5)
      return set_error(FIERRO_EINVAL, "fill %lld: tg_vortex reads statev(4)", (long long)f);
  }
  rc = validate_mesh_rz(mesh);
  if (rc) return rc;
  const int64_t nn = mesh->num_nodes, ne = mesh->num_elems, nsv = num_state_vars;
  const uint64_t* nie = mesh->nodes_in_elem;
  double* X = out->node_coords;
  double* V = out->node_vel;
  double* X1 = X + nn * 2;
  double* V1 = V + nn * 2;
  std::memcpy(X, mesh->coords, sizeof(double) * (size_t)nn * 2);
  std::memcpy(X1, mesh->coords, sizeof(double) * (size_t)nn * 2);
  std::memset(V, 0, sizeof(double) * (size_t)nn * 4);
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
  if (out->corner_force) std::memset(out->corner_force, 0, sizeof(double) * (size_t)ne * 8);
  double* vol = out->elem_vol;
  auto gather = [&](int64_t e, double x[4], double y[4]) {
    for (int l = 0; l < 4; ++l) {
      const double* c = X1 + nie[e * 4 + l] * 2;
      x[l] = c[0];
      y[l] = c[1];
    }
  };
  // get_vol (geometry.cpp:238-251)
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < ne; ++e) {
    double x[4], y[4];
    gather(e, x, y);
    vol[e] = vol_quad(x, y);
  }
  for (int64_t e = 0; e < ne; ++e)
    if (!(vol[e] > 0.0) || !std::isfinite(vol[e]))
      return set_error(FIERRO_ENUMERIC, "setup: element %lld has RZ volume %g (inverted, degenerate or below "
                       "the axis)", (long long)e, vol[e]);
  std::vector<int64_t> start, corners;
  node_corner_csr(nn, ne, nie, &start, &corners);
  std::vector<uint8_t> mask;
  std::vector<char> on_bdy;
  boundary_rz(mesh, boundaries, num_bcs, X1, start, corners, &mask, &on_bdy);
  const double PI = 3.141592653589793;
  // fills (setup.cpp:109-357) with the 2D centroid (z = 0)
  for (int64_t fi = 0; fi < num_fills; ++fi) {
    const fierro_mat_fill& F = fills[fi];
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < ne; ++e) {
      double ec[3] = {0.0, 0.0, 0.0};
      for (int l = 0; l < 4; ++l) {
        const double* c = X1 + nie[e * 4 + l] * 2;
        ec[0] += c[0];
        ec[1] += c[1];
        ec[2] = 0.0;
      }
      ec[0] = ec[0] / 4;
      ec[1] = ec[1] / 4;
      ec[2] = ec[2] / 4;
      const double radius = std::sqrt(ec[0] * ec[0] + ec[1] * ec[1] + ec[2] * ec[2]);
      const double radius_cyl = std::sqrt(ec[0] * ec[0] + ec[1] * ec[1]);
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
      const double gamma = sv[0], csmin = sv[1];
      out->elem_pres[e] = (gamma - 1.0) * out->elem_sie[ne + e] * out->elem_den[e];
      out->elem_sspd[e] = std::sqrt(gamma * (gamma - 1.0) * out->elem_sie[ne + e]);
      if (out->elem_sspd[e] < csmin) out->elem_sspd[e] = csmin;
      for (int l = 0; l < 4; ++l) {
        const uint64_t n = nie[e * 4 + l];
        const double* c = X1 + n * 2;
        double* v = V1 + n * 2;
        if (F.velocity == 0) {
          v[0] = F.u;
          v[1] = F.v;
        } else if (F.velocity == 1) {
          double dir[2] = {0.0, 0.0};
          double radius_val = 0.0;
          for (int d = 0; d < 2; ++d) {
            dir[d] = c[d];
            radius_val += c[d] * c[d];
          }
          radius_val = std::sqrt(radius_val);
          for (int d = 0; d < 2; ++d) {
            if (radius_val > 1.0e-14) dir[d] /= (radius_val);
            else dir[d] = 0.0;
          }
          v[0] = F.speed * dir[0];
          v[1] = F.speed * dir[1];
        } else if (F.velocity == 5) {
          v[0] = std::sin(PI * c[0]) * std::cos(PI * c[1]);
          v[1] = -1.0 * std::cos(PI * c[0]) * std::sin(PI * c[1]);
        }
      }
      if (F.velocity == 5) {
        out->elem_pres[e] = 0.25 * (std::cos(2.0 * PI * ec[0]) + std::cos(2.0 * PI * ec[1])) + 1.0;
        const double g4 = sv[4];
        out->elem_sie[ne + e] = out->elem_pres[e] / (F.den * (g4 - 1.0));
      }
    }
  }
  // boundary_velocity (setup.cpp:362)
  for (int64_t n = 0; n < nn; ++n)
    for (int d = 0; d < 2; ++d)
      if (mask[n] & (1u << d)) V1[n * 2 + d] = 0.0;
  // corner masses from Barlow's corner areas, node mass summed in corner order
  // (setup.cpp:365-420)
  std::vector<double> cmass((size_t)ne * 4);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < ne; ++e) {
    double x[4], y[4], ca[4];
    gather(e, x, y);
    corner_areas(x, y, ca);
    for (int l = 0; l < 4; ++l) cmass[e * 4 + l] = ca[l] * out->elem_den[e];
  }
#pragma omp parallel for schedule(static)
  for (int64_t n = 0; n < nn; ++n) {
    double m = 0.0;
    for (int64_t k = start[n]; k < start[n + 1]; ++k) m += cmass[corners[k]];
    out->node_mass[n] = m;
  }
  return FIERRO_OK;
}

}  // namespace rz
}  // namespace fierro
