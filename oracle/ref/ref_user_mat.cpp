// The test strength model handed to the reference through material_t's
// strength_model pointer (state.h:150-164), in the role of the reference's
// user_strength_model (user_mat.cpp:50-84), which is an empty stub.  Linked only
// into the reference oracle executables (oracle/build_ref.py); the deck keyword
// "strength <mat_id> <type>" of oracle/ref/ref_input.cpp selects it.
//
// Linear hypo-elasticity of the deviatoric stress without rotation terms, shear
// modulus G = statev(3):
//   D = (L + L^T) / 2,  D' = D - tr(D) / 3 I,
//   stress(1) = stress(0) + rk_alpha dt 2 G D'.
// The library's device hook (fierro_gb300/csrc/sgh_user_mat.cuh) and the C
// restatement (oracle/sgh_oracle.c) evaluate the same expressions in the same
// order, so the three agree bit for bit.
#include "matar.h"
#include "mesh.h"
#include "state.h"

void fierro_test_strength_model(const DViewCArrayKokkos<double>& elem_pres,
                                const DViewCArrayKokkos<double>& elem_stress, const size_t elem_gid,
                                const size_t mat_id, const DViewCArrayKokkos<double>& elem_state_vars,
                                const DViewCArrayKokkos<double>& elem_sspd, const double den, const double sie,
                                const ViewCArrayKokkos<double>& vel_grad,
                                const ViewCArrayKokkos<size_t>& elem_node_gids,
                                const DViewCArrayKokkos<double>& node_coords,
                                const DViewCArrayKokkos<double>& node_vel, const double vol, const double dt,
                                const double rk_alpha) {
  const double G = elem_state_vars(elem_gid, 3);
  double D[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) D[i][j] = 0.5 * (vel_grad(i, j) + vel_grad(j, i));
  const double tr = D[0][0] + D[1][1] + D[2][2];
  for (int i = 0; i < 3; ++i) D[i][i] -= tr / 3.0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      elem_stress(1, elem_gid, i, j) = elem_stress(0, elem_gid, i, j) + rk_alpha * dt * 2.0 * G * D[i][j];
}
