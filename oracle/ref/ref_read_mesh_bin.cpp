// Binary-mesh replacement for read_mesh_ensight (read_mesh.cpp:12-147), with the
// same signature and the same allocations, so generated meshes (jittered,
// permuted, 256^3) need no multi-GB ASCII .geo.  Linked only into the reference
// oracle build; the EnSight build links the reference's own read_mesh.cpp.
//
// File layout (little endian): "FSGHMESH", u64 num_nodes, u64 num_elems,
// f64 x[num_nodes], f64 y[num_nodes], f64 z[num_nodes] (no z for num_dims 2),
// u64 nodes_in_elem[num_elems][2^num_dims] (0-based).
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "mesh.h"
#include "state.h"

void read_mesh_ensight(char* MESH, mesh_t& mesh, node_t& node, elem_t& elem, corner_t& corner,
                       const size_t num_dims, const size_t rk_num_bins) {
  FILE* in = std::fopen(MESH, "rb");
  if (!in) {
    std::fprintf(stderr, "cannot open mesh %s\n", MESH);
    std::exit(2);
  }
  char magic[8];
  uint64_t nn = 0, ne = 0;
  if (std::fread(magic, 1, 8, in) != 8 || std::memcmp(magic, "FSGHMESH", 8) != 0 ||
      std::fread(&nn, 8, 1, in) != 1 || std::fread(&ne, 8, 1, in) != 1) {
    std::fprintf(stderr, "bad mesh header %s\n", MESH);
    std::exit(2);
  }
  mesh.initialize_nodes(nn);
  node.initialize(rk_num_bins, nn, num_dims);
  double* tmp = (double*)std::malloc(sizeof(double) * nn);
  for (size_t d = 0; d < num_dims; ++d) {
    if (std::fread(tmp, sizeof(double), nn, in) != nn) std::exit(2);
    for (size_t n = 0; n < nn; ++n) node.coords(0, n, d) = tmp[n];
  }
  std::free(tmp);
  mesh.initialize_elems(ne, num_dims);
  elem.initialize(rk_num_bins, nn, 3);  // sized by num_nodes, as read_mesh.cpp:106 does
  const size_t npe = num_dims == 2 ? 4 : 8;
  uint64_t* conn = (uint64_t*)std::malloc(sizeof(uint64_t) * ne * npe);
  if (std::fread(conn, sizeof(uint64_t), ne * npe, in) != ne * npe) std::exit(2);
  for (size_t e = 0; e < ne; ++e)
    for (size_t l = 0; l < npe; ++l) mesh.nodes_in_elem.host(e, l) = conn[e * npe + l];
  std::free(conn);
  mesh.nodes_in_elem.update_device();
  size_t num_corners = ne * mesh.num_nodes_in_elem;
  mesh.initialize_corners(num_corners);
  corner.initialize(num_corners, num_dims);
  for (size_t n = 0; n < nn; ++n)
    for (size_t rk = 1; rk < rk_num_bins; ++rk)
      for (size_t d = 0; d < num_dims; ++d) node.coords(rk, n, d) = node.coords(0, n, d);
  std::fclose(in);
}
