// User strength model: the role of the reference's user_strength_model
// (user_mat.cpp:50-84), compiled into the cycle kernels.  Replace the body of
// user_strength_model and rebuild the library to run another model; the call
// sites and the arguments stay.
//
// It runs once per element and RK stage for materials whose strength_type is
// 1 (hypo: in the force pass, after the corner forces, with the velocity
// gradient of the stage's input state; force_sgh.cpp:362-391) or 2 (hyper: in
// the element pass, after the density and before the EOS, with the velocity
// gradient of the state the stage produced; properties.cpp:46-95).  The force
// pass of the next stage uses the stress it leaves as tau = stress - p I
// (force_sgh.cpp:128-140).  Arguments:
//   stress1[9]  in/out: stress(1, e, i, j), row-major; on entry the value the
//               reference's stress(1) holds at the call (after rk_init on the
//               first stage)
//   stress0[9]  stress(0, e, i, j): the stress at the start of the cycle
//   L[9]        velocity gradient L(i, j) = d v_i / d x_j (momentum.cpp:59-144)
//   sv          element state variables: statev(e, k) is sv[k * sv_stride];
//               columns 0 and 1 (gamma, c_min) belong to the EOS and are read
//               from the copies taken at set_state, so a model keeps its
//               history in columns >= 2
//   mat_id, den, sie (elem_sie(e) as the reference passes it: bin 0, the
//   start of the cycle), vol, dt, rk_alpha
// The reference also hands the model the pressure and sound speed arrays; the
// ideal-gas EOS overwrites both after every stage, so they are not passed.
//
// The shipped model is linear hypo-elasticity of the deviatoric stress without
// rotation terms, shear modulus G = statev(3):
//   D = (L + L^T) / 2,  D' = D - tr(D) / 3 I,
//   stress1 = stress0 + rk_alpha dt 2 G D'.
// The oracle builds give the reference (oracle/ref/ref_user_mat.cpp, through
// material_t::strength_model) and the C restatement the same model, in the same
// operation order, so the three agree bit for bit in the exact mode.
#pragma once

// The number of state variables the model reads (statev(0) .. statev(3)); a
// handle with a strength material rejects a state with fewer.
constexpr int kUserStrengthStateVars = 4;

#ifdef __CUDACC__
__device__ __forceinline__ void user_strength_model(double* stress1, const double* stress0, const double* L,
                                                    double* sv, int sv_stride, int mat_id, double den, double sie,
                                                    double vol, double dt, double rk_alpha) {
  const double G = sv[3 * sv_stride];
  double D[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) D[i * 3 + j] = 0.5 * (L[i * 3 + j] + L[j * 3 + i]);
  const double tr = D[0] + D[4] + D[8];
  D[0] -= tr / 3.0;
  D[4] -= tr / 3.0;
  D[8] -= tr / 3.0;
#pragma unroll
  for (int k = 0; k < 9; ++k) stress1[k] = stress0[k] + rk_alpha * dt * 2.0 * G * D[k];
}
#endif
