// Mesh topology built on the GPU (sgh_topo.cu).
#ifndef FIERRO_SGH_TOPO_H
#define FIERRO_SGH_TOPO_H

#include "fierro_sgh.h"

struct fierro_sgh;

namespace fierro {
namespace topo {

// Fills the handle's device topology (d_nie, d_cin_start, d_cin, d_eie_start,
// d_eie, d_bc and the four renumbering maps; d_eie is allocated here) and the
// host renumbering maps (topo.node_int2ext, topo.elem_int2ext) from the caller's
// mesh, read by the GPU in place.  The boundary deck must be validated already.
int build_device(fierro_sgh* h, const fierro_mesh* mesh, const fierro_boundary* bcs, int64_t num_bcs);

}  // namespace topo
}  // namespace fierro

#endif
