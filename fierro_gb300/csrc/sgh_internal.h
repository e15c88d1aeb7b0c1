// Internal declarations shared by the host C++ and CUDA translation units of
// libfierro_sgh.  Not part of the public C ABI (include/fierro_sgh.h).
#ifndef FIERRO_SGH_INTERNAL_H
#define FIERRO_SGH_INTERNAL_H

#include <cstdint>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "fierro_sgh.h"

namespace fierro {

// Velocity components a boundary set holds at zero, as bits 0..dims-1
// (boundary.cpp:10-55): reflected zeroes the plane's normal component, fixed
// every component; the other kinds of bdy_hydro_conds (velocity, pressure,
// acceleration, contact; mesh.h:910-918) have no branch in boundary_velocity,
// so their nodes move freely.
inline unsigned char bc_mask_bits(int hydro_bc, int surface, int dims) {
  if (hydro_bc == 1) return (unsigned char)(1u << surface);
  if (hydro_bc == 0) return (unsigned char)((1u << dims) - 1u);
  return 0;
}

// An NVTX range around a C-ABI call: the call shows up by name on a profiler's
// timeline; without an attached tool the push and pop do nothing.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// Record an error for fierro_last_error() and return `code`.
int set_error(int code, const char* fmt, ...);
void clear_error();

// Host-side mesh topology in the device ("internal") numbering.
//
// Elements and nodes are renumbered along a Morton curve of their positions, for
// locality of the gathers.  Everything whose floating-point result depends on an
// order keeps the reference's order: each node's corner list is sorted by the
// caller's ("external") element id, which is the order in which
// update_velocity_sgh sums corner forces (mesh.h:218-241, momentum.cpp:31-41),
// and every element keeps its local node order 0..7.
struct HostTopo {
  int64_t nn = 0, ne = 0;
  std::vector<int64_t> node_int2ext, node_ext2int, elem_int2ext, elem_ext2int;
  std::vector<int32_t> nie;        // [ne][8] internal node ids of internal element e
  std::vector<int32_t> cin_start;  // [nn+1] corner CSR per internal node
  std::vector<int32_t> cin;        // internal corner ids e*8+lid, reference order
  std::vector<int32_t> eie_start;  // [ne+1] neighbour CSR (elements sharing a node)
  std::vector<int32_t> eie;
  std::vector<uint8_t> bc_mask;    // [nn] bit d: velocity component d held at zero
  int max_corners_per_node = 0;
  int npe = 8;                      // nodes per element: 8 hex, 4 quad (2D-RZ)
  // 2D-RZ: the boundary nodes (mesh.h:592-645) and their edge neighbours
  // (nodes_in_node, mesh.h:654-796), internal ids, for the axis mass fix
  std::vector<int32_t> axis_nodes, axis_nin_start, axis_nin;
};

// Indices of n points [n][3] in Morton order (21 bits per axis on the bounding
// box; a stable sort, so equal keys keep their index order).
std::vector<int64_t> morton_order(const double* pts, int64_t n);

// The mesh's num_dims: 3 (hex) or 2 (2D-RZ quads); 0 reads as 3.
inline int mesh_dims(const fierro_mesh* m) { return (m && m->num_dims == 2) ? 2 : 3; }

// Null pointers, num_dims, sizes and the 32-bit index limit of a mesh (no
// per-element checks).
int check_mesh_header(const fierro_mesh* mesh);
// 2D-RZ counterparts (sgh_rz.cpp): boundary deck checks and topology.
int validate_bcs_rz(const fierro_boundary* bcs, int64_t num_bcs);
int build_topology_rz(const fierro_mesh* mesh, const fierro_boundary* bcs, int64_t num_bcs, HostTopo* t);
// Surface tags and condition kinds of a boundary deck.
int validate_bcs(const fierro_boundary* bcs, int64_t num_bcs);

// Validates the mesh and boundary deck and fills `t`.  `renumber` = false keeps
// the caller's numbering (identity maps).
int build_topology(const fierro_mesh* mesh, const fierro_boundary* bcs, int64_t num_bcs, bool renumber,
                   HostTopo* t);

// The boundary-condition bit mask per external node from the boundary patches
// (faces owned by one element) that lie on each boundary set's surface
// (setup.cpp:431-665).
int boundary_masks(const fierro_mesh* mesh, const fierro_boundary* bcs, int64_t num_bcs,
                   const double* coords_bin1, std::vector<uint8_t>* mask_ext,
                   std::vector<std::vector<int64_t>>* set_nodes);

}  // namespace fierro

#endif
