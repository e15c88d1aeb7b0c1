/* CPU oracle for the SGH cycle: a plain-C restatement of Fierro's
 * Explicit-Lagrange-Kokkos/SGH_solver 3D hex path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py may load it, and only as the checker.  The GB300
 * library never links or calls it.
 *
 * Every function follows the reference arithmetic operation by operation (same
 * operands, same association order, libm pow/sqrt), so with
 * -ffp-contract=off it reproduces the reference's doubles bit for bit; the
 * per-function comments cite the reference file:line restated.
 *
 * Arrays crossing this interface use the reference layouts:
 *   node_coords, node_vel  [2][num_nodes][3]   (rk bin, node, dim)
 *   elem_sie               [2][num_elems]
 *   elem_stress            [2][num_elems][3][3]
 *   elem_statev            [num_elems][num_state_vars]
 *   corner_force           [8*num_elems][3]    corner gid = elem*8 + node_lid
 *   nodes_in_elem          [num_elems][8]      0-based, hex ordering of mesh.h:15-45
 */
#ifndef FIERRO_SGH_ORACLE_H
#define FIERRO_SGH_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* material_t (state.h:130-178); the ideal-gas EOS only.  strength_type 1 (hypo)
 * and 2 (hyper) run the test strength model of oracle/ref/ref_user_mat.cpp
 * (shear modulus statev(3); needs num_state_vars >= 4). */
typedef struct {
  int eos_model;      /* 0 = ideal_gas (eos.cpp:12) */
  int strength_type;  /* model::strength_tag (state.h:107-112): 0 none, 1 hypo, 2 hyper */
  double q1, q1ex, q2, q2ex;
} orc_material;

/* boundary_t (mesh.h:924-935) */
typedef struct {
  int surface;   /* bdy::bdy_tag: 0 x-plane, 1 y-plane, 2 z-plane, 3 cylinder, 4 sphere */
  double value;
  int hydro_bc;  /* bdy::bdy_hydro_conds: 0 fixed, 1 reflected */
} orc_boundary;

/* mat_fill_t (mesh.h:858-890) */
typedef struct {
  int volume;    /* region::vol_tag: 0 global, 1 box, 2 cylinder, 3 sphere */
  int mat_id;
  double x1, x2, y1, y2, z1, z2;
  double radius1, radius2;
  int velocity;  /* init_conds: 0 cartesian, 1 radial, 2 spherical, 5 tg_vortex */
  double u, v, w, speed, sie, den;
} orc_fill;

/* The scalar controls of sgh_solve (mesh.h:1175-1208, driver.cpp:35-62). */
typedef struct {
  double time_final, dt_max, dt_min, dt_cfl, dt_start;
  double graphics_dt_ival;
  int64_t graphics_cyc_ival;
  int64_t cycle_stop;
  int64_t rk_num_stages;
  double fuzz, tiny, small;
} orc_params;

enum orc_array {
  ORC_NODE_COORDS = 0, ORC_NODE_VEL, ORC_NODE_MASS,
  ORC_ELEM_DEN, ORC_ELEM_PRES, ORC_ELEM_STRESS, ORC_ELEM_SSPD, ORC_ELEM_SIE,
  ORC_ELEM_VOL, ORC_ELEM_DIV, ORC_ELEM_MASS, ORC_ELEM_MAT_ID, ORC_ELEM_STATEV,
  ORC_CORNER_FORCE, ORC_BDY_NODE_MASK, ORC_NUM_ARRAYS
};

typedef struct orc_sim orc_sim;

orc_sim* orc_create(int64_t num_nodes, int64_t num_elems, const int64_t* nodes_in_elem,
                    const double* coords /* [num_nodes][3] */);
void orc_destroy(orc_sim* s);

int orc_set_materials(orc_sim* s, int num_materials, const orc_material* m,
                      int num_state_vars, const double* state_vars /* [nmat][nsv] */);
int orc_set_boundaries(orc_sim* s, int num_bcs, const orc_boundary* b);
/* setup.cpp:10-424 (plus get_vol at driver.cpp:239 first). */
int orc_setup(orc_sim* s, int num_fills, const orc_fill* fills);

/* Reset time_value=0, dt=dt_start, graphics_time=graphics_dt_ival (driver.cpp:270-274). */
void orc_init_time(orc_sim* s, const orc_params* p);
/* Advance by whole cycles of sgh_solve's loop (sgh_solve.cpp:125-634).  Stops early
 * when time reaches time_final.  Returns the number of cycles run. */
int64_t orc_run_cycles(orc_sim* s, const orc_params* p, int64_t ncycles);
/* Advance by single RK stages (for per-kernel checks).  A stage at the start of a
 * cycle first runs get_timestep and rk_init. */
int64_t orc_run_stages(orc_sim* s, const orc_params* p, int64_t nstages);

/* The diagnostic tallies of sgh_solve.cpp:77-101 (summed in index order). */
void orc_energy(const orc_sim* s, double* ie, double* ke);
void orc_time(const orc_sim* s, double* time_value, double* dt, double* graphics_time,
              int64_t* cycle);

/* Copy one state array in/out in the reference layout; returns the element count. */
int64_t orc_get(const orc_sim* s, int which, void* out);
int64_t orc_set(orc_sim* s, int which, const void* in);

/* Geometry kernels exposed for known-answer tests (geometry.cpp:40-310). */
void orc_bmatrix(const double x[8], const double y[8], const double z[8], double B[8][3]);
double orc_vol_hex(const double x[8], const double y[8], const double z[8]);

/* ---- 2D-RZ (num_dims == 2), oracle/sgh_oracle_rz.c --------------------------
 * The same calls for quad meshes: coordinates [num_nodes][2] (x axial, y
 * radial), nodes_in_elem [num_elems][4], and in orc_rz_get / orc_rz_set
 * node_coords / node_vel [2][Nn][2] and corner_force [4Ne][2].  Materials
 * accept strength_type 0 and 1 (hyper is refused); boundaries accept x and y
 * planes and cylinders (fixed); fills refuse the spherical velocity. */
typedef struct orc_rz orc_rz;
orc_rz* orc_rz_create(int64_t num_nodes, int64_t num_elems, const int64_t* nodes_in_elem,
                      const double* coords);
void orc_rz_destroy(orc_rz* s);
int orc_rz_set_materials(orc_rz* s, int num_materials, const orc_material* m, int num_state_vars,
                         const double* state_vars);
int orc_rz_set_boundaries(orc_rz* s, int num_bcs, const orc_boundary* b);
int orc_rz_setup(orc_rz* s, int num_fills, const orc_fill* fills);
void orc_rz_init_time(orc_rz* s, const orc_params* p);
int64_t orc_rz_run_cycles(orc_rz* s, const orc_params* p, int64_t ncycles);
int64_t orc_rz_run_stages(orc_rz* s, const orc_params* p, int64_t nstages);
void orc_rz_energy(const orc_rz* s, double* ie, double* ke);
void orc_rz_time(const orc_rz* s, double* time_value, double* dt, double* graphics_time, int64_t* cycle);
int64_t orc_rz_get(const orc_rz* s, int which, void* out);
int64_t orc_rz_set(orc_rz* s, int which, const void* in);
void orc_rz_bmatrix(const double x[4], const double y[4], double B[4][2]);
double orc_rz_vol_quad(const double x[4], const double y[4]);
double orc_rz_area_quad(const double x[4], const double y[4]);
void orc_rz_corner_areas(const double x[4], const double y[4], double ca[4]);

#ifdef __cplusplus
}
#endif
#endif
