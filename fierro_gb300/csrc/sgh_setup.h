// The initial state computed on the GPU (sgh_setup.cu) for fierro_sgh_setup.
#ifndef FIERRO_SGH_SETUP_H
#define FIERRO_SGH_SETUP_H

#include "fierro_sgh.h"

namespace fierro {
namespace setup_gpu {

// True when the GPU set-up applies: kernels can read the caller's host arrays
// and no fill asks for the tg_vortex velocity (libm sin / cos, host only).
bool usable(const fierro_mat_fill* fills, int64_t num_fills);
// The set-up of fierro_sgh_setup on the GPU; the arguments are validated by the
// caller apart from the per-element mesh checks, which run here.
int run(const fierro_mesh* mesh, const double* state_vars, int64_t num_state_vars, const fierro_mat_fill* fills,
        int64_t num_fills, const fierro_boundary* boundaries, int64_t num_bcs, fierro_sgh_state* out);

}  // namespace setup_gpu
}  // namespace fierro

#endif
