// 2D-RZ (axisymmetric, num_dims == 2) path: per-launch argument records of the
// quad kernels (sgh_rz_kernels.cu) and the host entry points the C ABI
// dispatches to for a handle created from a quad mesh (sgh_rz.cpp).
//
// HBM layout (internal, Morton-ordered numbering), besides the 3D handle's
// element fields: nodes x, y (x axial, y radial) and u, v in two ping-pong bins,
// half velocity hx, hy, the radius each node had at the start of the stage
// (the energy's node_radius, energy_sgh.cpp:33-36), the areal node mass and the
// extensive node mass m*y fixed at set_state (sgh_solve.cpp:106-114); int32
// nodes_in_elem [ne][4]; corner forces [8][ne] (row lid*2+dim); the boundary
// nodes with their edge neighbours for the axis mass fix.
#ifndef FIERRO_SGH_RZ_H
#define FIERRO_SGH_RZ_H

#include <cuda_runtime.h>

#include "fierro_sgh.h"
#include "sgh_device.h"

struct fierro_sgh;

namespace fierro {

struct RzForceArgs {
  int ne;
  const int* nie;
  const int* eie_start;
  const int* eie;
  const int* mat;
  const double* qtab;           // [nmat][4] = q1, q1ex, q2, q2ex
  const double *x, *y, *u, *v;  // the stage's input state (reference bin 1)
  const double *den, *pres, *sspd, *vol;
  const double* div;            // this stage's divergence (previous element pass)
  double* force;                // [8][ne]
  const Ctrl* ctrl;
  double fuzz, small;
  // hypo strength materials (stress rows [9][ne]), as in ForceArgs
  const double* stress_cur;
  const double* stress0;
  double* stress_out;
  const int* stype;
  double* statev;
  const double* sie0;
  double rk_alpha;
  int copy_stress;
};

struct RzNodeArgs {
  int nn, ne;
  const int* cin_start;
  const int* cin;                       // internal corner ids e*4+lid, reference order
  const double* force;
  double* node_mass;                    // read (this stage), then the areal mass of the new position
  const double* node_ext;               // extensive node mass m*y
  const unsigned char* bc_mask;
  const double *u0, *v0, *x0, *y0;      // cycle start (reference bin 0)
  double *u1, *v1, *x1, *y1;            // updated (reference bin 1)
  const double* yin;                    // radius at the start of the stage (bin 0 on the first stage)
  double *hx, *hy, *rad;
  const Ctrl* ctrl;
  double rk_alpha, tiny;
};

struct RzAxisArgs {
  int naxis;
  const int* nodes;      // boundary nodes (mesh.h:592-645)
  const int* nin_start;  // their edge neighbours (mesh.h:654-796)
  const int* nin;
  const double* y1;
  double* node_mass;
  const Ctrl* ctrl;
  double tiny;
};

// kind: 0 = stage update, 1 = last stage (adds the CFL partial minima),
// 2 = prime (divergence and CFL of an uploaded state only).
struct RzElemArgs {
  int ne;
  const int* nie;
  const double *x, *y, *u, *v;  // updated state
  const double *hx, *hy, *rad;
  const double* force;
  const double* mass;
  const double* sie0;
  double* sie1;
  const double *gamma, *csmin;
  double *den, *pres, *sspd, *vol;
  double* div;  // divergence for the next stage
  long long* cfl_part;
  Ctrl* ctrl;
  double rk_alpha, dt_cfl, fuzz;
};

struct RzEnergyArgs {
  int ne, nn;
  const double *mass, *sie;
  const double *node_mass, *u, *v, *y;
  double* part;  // [2][nblocks]
  double* out;   // [2]
};

struct RzKernelSet {
  void (*force)(const RzForceArgs&, cudaStream_t);
  void (*node)(const RzNodeArgs&, cudaStream_t);
  void (*axis)(const RzAxisArgs&, cudaStream_t);
  void (*elem)(const RzElemArgs&, int kind, cudaStream_t);
  void (*ext_mass)(int nn, const double* node_mass, const double* y, double* ext, cudaStream_t);
  void (*energy)(const RzEnergyArgs&, cudaStream_t);
};

const RzKernelSet& rz_kernels_exact();
const RzKernelSet& rz_kernels_fma();

namespace rz {

// The C ABI's per-handle operations for a quad mesh (sgh_rz.cpp).
int create(fierro_sgh* h, const fierro_mesh* mesh, const fierro_material* materials, int64_t num_materials,
           const fierro_boundary* boundaries, int64_t num_bcs);
int set_state(fierro_sgh* h, const fierro_sgh_state* s);
int prime(fierro_sgh* h);
int get_state(fierro_sgh* h, fierro_sgh_state* s, const int bins[2], int div_buffer);
// Enqueues RK stage s of a cycle whose start state is in bin c; with `ev`, an
// event is recorded after each launch.
int enqueue_stage(fierro_sgh* h, int c, int s, cudaEvent_t* ev, size_t* k);
int energy(fierro_sgh* h, int bin, double* ie, double* ke);
// setup (setup.cpp:10-424) with num_dims == 2, in the caller's numbering.
int setup(const fierro_mesh* mesh, const fierro_material* materials, int64_t num_materials,
          const double* state_vars, int64_t num_state_vars, const fierro_mat_fill* fills, int64_t num_fills,
          const fierro_boundary* boundaries, int64_t num_bcs, fierro_sgh_state* out);

}  // namespace rz
}  // namespace fierro

#endif
