/* fierro_sgh.h -- C ABI of the GB300-native SGH (staggered-grid hydrodynamics)
 * Lagrangian cycle for unstructured 3D hexahedral meshes.
 *
 * Drop-in boundary for Fierro's Explicit-Lagrange-Kokkos/SGH_solver hot path:
 * the record types mirror material_t / boundary_t / mat_fill_t
 * (state.h:130-178, mesh.h:858-935), state arrays use the reference layouts, and
 * fierro_sgh_solve / fierro_sgh_setup replace sgh_solve / setup
 * (mesh.h:1175-1208, mesh.h:1006-1028).  Plain pointers and sizes only.
 *
 * Reference layouts of state arrays (all host memory, float64 unless noted):
 *   node_coords, node_vel   [2][num_nodes][3]      (rk bin, node, dim)
 *   node_mass               [num_nodes]
 *   elem_den, elem_pres, elem_sspd, elem_vol, elem_div, elem_mass   [num_elems]
 *   elem_sie                [2][num_elems]
 *   elem_stress             [2][num_elems][3][3]
 *   elem_mat_id             [num_elems]            (uint64 = size_t)
 *   elem_statev             [num_elems][num_state_vars]   statev(0)=gamma, (1)=c_min
 *   corner_force            [8*num_elems][3]       corner gid = elem*8 + node_lid
 *   nodes_in_elem           [num_elems][8]         (uint64, 0-based, mesh.h:15-45 order)
 *
 * Errors: every call returns FIERRO_OK (0) or a FIERRO_E* code; the library never
 * exits the process.  fierro_last_error() returns the text of the calling thread's
 * last error.  A handle is used by one host thread at a time.
 */
#ifndef FIERRO_SGH_H
#define FIERRO_SGH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FIERRO_OK 0
#define FIERRO_EINVAL 1     /* bad argument, mesh or deck */
#define FIERRO_ENOMEM 2     /* device or host allocation failed */
#define FIERRO_ECUDA 3      /* CUDA runtime error */
#define FIERRO_ENUMERIC 4   /* non-positive volume or non-finite state detected */
#define FIERRO_ETIMEDOUT 5  /* a bounded device wait gave up */
#define FIERRO_ENOTSUP 6    /* valid in the reference but outside this path */

/* Arithmetic modes of the device kernels. */
#define FIERRO_FP_EXACT 0   /* reference operation order, no contraction: doubles
                               match the reference's uncontracted evaluation */
#define FIERRO_FP_FMA 1     /* same schedule with fused multiply-adds and
                               reciprocal reuse (differs in the last bits) */

/* material_t (state.h:130-178).  eos_model 0 = ideal_gas (eos.cpp:12).
 * strength_type (model::strength_tag, state.h:103-113): 0 none, 1 hypo (the
 * stress model runs in the force pass, force_sgh.cpp:362-391), 2 hyper (in the
 * state update, properties.cpp:46-95).  The model is the library's compiled-in
 * user_strength_model (fierro_gb300/csrc/sgh_user_mat.cuh), the counterpart of
 * the reference's user_mat.cpp function pointer; the shipped one is linear
 * hypo-elasticity with shear modulus statev(3).  A handle with a strength
 * material carries the full stress tensor (both bins) and all state variables
 * on the device and needs num_state_vars >= 4. */
typedef struct {
  int eos_model;
  int strength_type;
  double q1, q1ex, q2, q2ex;
} fierro_material;

/* boundary_t (mesh.h:924-935).  surface: 0 x-plane, 1 y-plane, 2 z-plane,
 * 3 cylinder, 4 sphere.  hydro_bc (bdy_hydro_conds, mesh.h:910-918): 0 fixed,
 * 1 reflected (planes only); 2 velocity, 3 pressure, 4 acceleration, 5 contact
 * are accepted and, as in the reference's boundary_velocity (boundary.cpp:10-55),
 * hold no velocity component. */
typedef struct {
  int surface;
  double value;
  int hydro_bc;
} fierro_boundary;

/* mat_fill_t (mesh.h:858-890).  volume: 0 global, 1 box, 2 cylinder, 3 sphere.
 * velocity: 0 cartesian, 1 radial, 2 spherical, 5 tg_vortex. */
typedef struct {
  int volume;
  int mat_id;
  double x1, x2, y1, y2, z1, z2;
  double radius1, radius2;
  int velocity;
  double u, v, w, speed, sie, den;
} fierro_mat_fill;

/* The scalar controls of sgh_solve (mesh.h:1175-1208; defaults driver.cpp:35-62). */
typedef struct {
  double time_final, dt_max, dt_min, dt_cfl, dt_start;
  double graphics_dt_ival;
  int64_t graphics_cyc_ival;
  int64_t cycle_stop;
  int64_t rk_num_stages;
  double fuzz, tiny, small;
} fierro_sgh_params;

/* Mesh: num_nodes, num_elems and nodes_in_elem (mesh_t, mesh.h:68-817) plus the
 * initial coordinates (node_coords bin 1 after read_mesh_ensight) and
 * mesh_t::num_dims.  num_dims 3 (or 0): hexes, nodes_in_elem [Ne][8], coords
 * [Nn][3].  num_dims 2: the 2D-RZ (axisymmetric) path, quads nodes_in_elem
 * [Ne][4] counter-clockwise, coords [Nn][2] = (x axial, y radial); the state
 * arrays then hold 2 components per node (node_coords, node_vel [2][Nn][2],
 * corner_force [4Ne][2]).  On the 2D-RZ path: boundary surfaces x-plane,
 * y-plane and cylinder (the reference's z-plane and sphere read a third
 * coordinate 2D arrays do not have); no hyper strength models (update_state2D,
 * properties.cpp:146-160, writes 3D normals into a 2D array); no spherical
 * velocity fill (setup.cpp:272-296 reads a third coordinate); state transfers
 * through the host; no graphics dumps, adjoint, batch or device view. */
typedef struct {
  int64_t num_nodes;
  int64_t num_elems;
  const uint64_t* nodes_in_elem;
  const double* coords;
  int64_t num_dims;
} fierro_mesh;

/* Host state in the reference layouts (see top of file).  For set_state the
 * fields marked (in) are required; for get_state any NULL field is skipped. */
typedef struct {
  double* node_coords;   /* (in) [2][Nn][3] */
  double* node_vel;      /* (in) [2][Nn][3] */
  double* node_mass;     /* (in) [Nn] */
  double* elem_den;      /* (in) [Ne] */
  double* elem_pres;     /* (in) [Ne] */
  double* elem_stress;   /* [2][Ne][3][3]; NULL reads as zero.  Without a strength
                            material it must be zero; with one it is carried and
                            returned by get_state */
  double* elem_sspd;     /* (in) [Ne] */
  double* elem_sie;      /* (in) [2][Ne] */
  double* elem_vol;      /* (in) [Ne] */
  double* elem_div;      /* [Ne] (recomputed by the first stage) */
  double* elem_mass;     /* (in) [Ne] */
  uint64_t* elem_mat_id; /* (in) [Ne] */
  double* elem_statev;   /* (in) [Ne][num_state_vars]; get_state returns it on a
                            handle with a strength material (the model may
                            update columns >= 2) */
  double* corner_force;  /* [8Ne][3] (output of the last stage) */
  int64_t num_state_vars;
} fierro_sgh_state;

typedef struct fierro_sgh fierro_sgh;

/* Text of the calling thread's last error ("" if none). */
const char* fierro_last_error(void);
/* Library version string. */
const char* fierro_version(void);

/* setup (setup.cpp:10-424) with get_vol first (driver.cpp:239), on the host:
 * boundary tagging, fills, EOS, velocity ICs, BCs and node mass.  Writes the
 * initial state (bin 1 and bin 0 as the reference leaves them) into `out`.
 * state_vars is [num_materials][num_state_vars]. */
int fierro_sgh_setup(const fierro_mesh* mesh, const fierro_material* materials, int64_t num_materials,
                     const double* state_vars, int64_t num_state_vars,
                     const fierro_mat_fill* fills, int64_t num_fills,
                     const fierro_boundary* boundaries, int64_t num_bcs, fierro_sgh_state* out);

/* sgh_solve (sgh_solve.cpp:8-692): run the cycle loop on the GPU from the state
 * in `state` (host, reference layouts) and write the final state back.  On
 * entry *time_value, *graphics_time and dt are the loop's starting values; on
 * return *time_value and *graphics_time hold the final ones and, when non-NULL,
 * *cycles_run the number of cycles executed.  Host<->device copies are part of
 * the call.  fp_mode is FIERRO_FP_EXACT or FIERRO_FP_FMA. */
int fierro_sgh_solve(const fierro_mesh* mesh, const fierro_material* materials, int64_t num_materials,
                     const fierro_boundary* boundaries, int64_t num_bcs, fierro_sgh_state* state,
                     double* time_value, double time_final, double dt_max, double dt_min, double dt_cfl,
                     double* graphics_time, int64_t graphics_cyc_ival, double graphics_dt_ival,
                     int64_t cycle_stop, int64_t rk_num_stages, double dt, double fuzz, double tiny,
                     double small, int fp_mode, int64_t* cycles_run);

/* ---- persistent handle: device-resident mesh and state ---------------------
 * create: builds the device mesh (Morton-renumbered; reference summation orders
 * kept), boundary node sets and materials.  stream may be NULL (the handle then
 * owns a stream) or a cudaStream_t the caller owns. */
int fierro_sgh_create(const fierro_mesh* mesh, const fierro_material* materials, int64_t num_materials,
                      const fierro_boundary* boundaries, int64_t num_bcs, const fierro_sgh_params* params,
                      int fp_mode, void* stream, fierro_sgh** out);
int fierro_sgh_destroy(fierro_sgh* h);
/* Upload a state (reference layouts) and reset time_value=0, dt=dt_start,
 * graphics_time=graphics_dt_ival, cycle=0. */
int fierro_sgh_set_state(fierro_sgh* h, const fierro_sgh_state* state);
int fierro_sgh_get_state(fierro_sgh* h, fierro_sgh_state* state);
/* Enqueue up to `cycles` cycles on the handle's stream without waiting.  The
 * loop stops by itself once time_value reaches time_final (the remaining
 * enqueued cycles do nothing). */
int fierro_sgh_enqueue_cycles(fierro_sgh* h, int64_t cycles);
/* Run `cycles` cycles and wait; *cycles_run (if non-NULL) = cycles executed. */
int fierro_sgh_run(fierro_sgh* h, int64_t cycles, int64_t* cycles_run);
/* Run single RK stages (a stage at a cycle start first computes dt). */
int fierro_sgh_run_stages(fierro_sgh* h, int64_t stages);
int fierro_sgh_synchronize(fierro_sgh* h);
/* Loop scalars: time_value, dt of the last cycle, graphics_time, cycles done. */
int fierro_sgh_time(fierro_sgh* h, double* time_value, double* dt, double* graphics_time, int64_t* cycle);
/* Energy tallies of sgh_solve.cpp:77-101: IE = sum M e, KE = 1/2 sum m |v|^2
 * (deterministic device reductions). */
int fierro_sgh_energy(fierro_sgh* h, double* ie, double* ke);
/* Run `cycles` cycles with a CUDA event recorded after every launch and wait.
 * kernel_ms[i] (array of fierro_sgh_launches_per_cycle entries, may be NULL)
 * receives the device time summed over the cycles of launch slot i of a cycle
 * (slot 0 = dt, then force/node/elem per stage, last = end-of-cycle); *total_ms
 * receives the device time from the first launch to the last.  Same results as
 * fierro_sgh_run. */
int fierro_sgh_run_timed(fierro_sgh* h, int64_t cycles, float* kernel_ms, float* total_ms, int64_t* cycles_run);
/* Number of kernel launches one cycle enqueues (for launch accounting). */
int64_t fierro_sgh_launches_per_cycle(const fierro_sgh* h);

/* Checkpoint / restart (no counterpart in the reference, which can only call
 * sgh_solve again from the state it left, restarting dt from dt_start).
 * fierro_sgh_checkpoint writes, at a cycle boundary, everything the cycle loop
 * carries into the next cycle (both state bins, the corner normals, divergences
 * and CFL partial minima the next stage and dt step read, masses, stress and
 * state variables, the loop scalars) to a file, with a fingerprint of the
 * device topology.  fierro_sgh_restart loads it into a handle created from the
 * same mesh, deck and parameters (FIERRO_EINVAL otherwise); the loop then
 * continues bit for bit as if it had not stopped.  Graphics-dump and adjoint
 * state are not part of a checkpoint. */
int fierro_sgh_checkpoint(fierro_sgh* h, const char* path);
int fierro_sgh_restart(fierro_sgh* h, const char* path);

/* Checks the handle's device topology against the invariants the cycle kernels
 * rely on (node ids in range and distinct per element; corner lists complete,
 * each corner once, in the reference's summation order; neighbours share a
 * node; boundary masks; 2D-RZ axis lists), on the GPU, range-checking every
 * index before use.  FIERRO_OK, or FIERRO_EINVAL naming the first failing
 * check.  A stand-in for a memory checker, which is not available here. */
int fierro_sgh_validate(fierro_sgh* h);

/* Health word of the run since set_state (the device writes it, never traps):
 * FIERRO_HEALTH_BAD_VOLUME and FIERRO_HEALTH_BAD_STATE also make the run calls
 * return FIERRO_ENUMERIC; FIERRO_HEALTH_DT_FLOOR is a warning: some element's CFL
 * step fell below dt_min, and the time step was raised to dt_min as the
 * reference's clamp does (time_integration.cpp:131-135), so the run may be
 * unstable. */
#define FIERRO_HEALTH_BAD_VOLUME 1u
#define FIERRO_HEALTH_BAD_STATE 2u
#define FIERRO_HEALTH_DT_FLOOR 4u
int fierro_sgh_status(fierro_sgh* h, uint32_t* flags);
/* Bytes of device memory the handle holds. */
int64_t fierro_sgh_device_bytes(const fierro_sgh* h);

/* ---- batched ensemble: many independent problems advanced together ---------
 * All instances' meshes and states live in one device layout and every kernel
 * of a cycle covers all of them in one launch; each instance keeps its own dt,
 * time, CFL number, materials, boundaries and stop time.  Results per instance
 * equal those of a separate fierro_sgh handle bit for bit.  rk_num_stages, fuzz,
 * tiny and small must be equal across instances.  No counterpart in the
 * reference (it runs one problem per process). */
typedef struct {
  fierro_mesh mesh;
  const fierro_material* materials;
  int64_t num_materials;
  const fierro_boundary* boundaries;
  int64_t num_bcs;
  fierro_sgh_params params;
} fierro_batch_instance;

typedef struct fierro_batch fierro_batch;

int fierro_batch_create(const fierro_batch_instance* instances, int64_t num_instances, int fp_mode, void* stream,
                        fierro_batch** out);
int fierro_batch_destroy(fierro_batch* b);
/* Upload instance i's initial state (reference layouts).  Every instance needs a
 * state before the first fierro_batch_run; states cannot be replaced after it. */
int fierro_batch_set_state(fierro_batch* b, int64_t instance, const fierro_sgh_state* state);
int fierro_batch_get_state(fierro_batch* b, int64_t instance, fierro_sgh_state* state);
/* Run `cycles` cycles of every instance (one CUDA graph launch per cycle) and
 * wait; instances that reach their time_final stop by themselves. */
int fierro_batch_run(fierro_batch* b, int64_t cycles);
int fierro_batch_time(fierro_batch* b, int64_t instance, double* time_value, double* dt, int64_t* cycle);
int64_t fierro_batch_num_instances(const fierro_batch* b);
int64_t fierro_batch_device_bytes(const fierro_batch* b);

/* Launch shape of a batch's cycle kernels (no counterpart in the reference):
 * threads per block of the corner-force, node and element passes (powers of two;
 * force and element 32..128, node 32..1024), and `persistent`: 0 = one block per
 * tile of elements or nodes, p = 1..8 = a persistent grid that fills every SM p
 * times over with the kernel's resident blocks and loops over the tiles.
 * `fused_stage` 1 runs each RK stage as ONE cooperative launch of elem_block
 * threads per block over the resident grid (force pass, grid barrier, node pass,
 * grid barrier, element pass; the other blocks and `persistent` are then
 * unused).  Results do not depend on the shape (every element and node runs the
 * same arithmetic; the CFL minimum is order-independent).
 * Default {128, 256, 128, 0, 0}. */
typedef struct {
  int force_block;
  int node_block;
  int elem_block;
  int persistent;
  int fused_stage;
} fierro_batch_shape;

/* Set or read the shape; set only before the first fierro_batch_run. */
int fierro_batch_set_shape(fierro_batch* b, const fierro_batch_shape* shape);
int fierro_batch_get_shape(const fierro_batch* b, fierro_batch_shape* shape);
/* Autotuner: after every instance has its state and before the first run, time
 * `cycles` cycles (after one warm-up cycle) of the captured cycle graphs for each
 * candidate shape of a coordinate descent over the force block {128, 64, 32}, the
 * node block {256, 128, 512, 64}, the element block {128, 64, 32}, the
 * persistent grid {0, 1, 2} and the fused stage at the chosen element block,
 * each from the uploaded state (saved and restored on the device; needs one
 * extra copy of the batch's state), and keep the fastest.  The state afterwards
 * is the uploaded one.  fierro_batch_run returns FIERRO_ETIMEDOUT if a fused
 * stage's grid barrier gave up waiting (its wait is bounded). */
int fierro_batch_autotune(fierro_batch* b, int64_t cycles, fierro_batch_shape* chosen);
/* The last autotune's candidates in timing order and their ms per cycle. */
int fierro_batch_tune_log(const fierro_batch* b, fierro_batch_shape* shapes, double* ms_per_cycle, int64_t capacity,
                          int64_t* count);

/* Energy tallies IE = sum elem_mass*elem_sie and KE = 1/2 sum node_mass*|v|^2
 * over device arrays the caller owns, enqueued on `stream` (NULL = default
 * stream), written as two doubles to the DEVICE pointer ie_ke.  No counterpart in
 * the reference: it exists for callers that cannot call cudaMalloc when they
 * need the tallies (for example while capturing a CUDA graph, or when all device
 * memory belongs to the caller's own arena), and it allocates nothing.  Its
 * scratch is an 8 KiB array held by every GPU that loads the library until the
 * process exits; at most 2^30 elements and 2^30 nodes per call (EINVAL beyond).
 * The first call in each CUDA context (the device's primary context, again after
 * a cudaDeviceReset, or a context of the caller's own) looks up that array's
 * device address in that context, so make the first call in a context before
 * any stream capture in it.  All calls share the array: calls that overlap on
 * the GPU race on it. */
int fierro_energy_tally_noalloc(const double* elem_mass, const double* elem_sie, int64_t num_elems,
                                const double* node_mass, const double* node_u, const double* node_v,
                                const double* node_w, int64_t num_nodes, double* ie_ke, void* stream);

/* FP64 roof calibration on the current device: dependent-chain-free DFMA
 * throughput, in fused multiply-adds per second (one FMA = 2 FLOP). */
int fierro_measure_fp64_rate(double* dfma_per_second);
/* FP64 pipe survey on the current device (no counterpart in the reference): a
 * pure stream of `chains` (1, 2, 4, 8, 16) independent chains per thread of one
 * operation (op 0 fma, 1 add, 2 mul), `threads` per block, `blocks_per_sm`
 * blocks per SM; operations per second, best of two timed launches. */
int fierro_fp64_stream_rate(int chains, int op, int threads, int blocks_per_sm, double* ops_per_second);
/* The arithmetic mode's square root (which 0), cube root (1), quotient (2) or
 * reciprocal (3) against the CUDA library's, on the current device (no
 * counterpart in the reference): n inputs, eight special values (zero, -0, the
 * smallest subnormal, infinity, NaN, -1, the largest and smallest normal
 * double; the divisor for a quotient) then seeded 2^E (1 + f), E uniform in
 * [lo_exp, hi_exp] (within -1022..1023), f's 52 bits uniform (quotients: two such
 * operands of random signs).  which 4, 5, 6: the square root, quotient and
 * reciprocal on arguments whose exact result lies just off a rounding boundary
 * (the hard cases of correct rounding); which 7, 8: the adjoint's ~2^-43
 * reciprocal and reciprocal square root against 1 / x and 1 / sqrt(x).
 * out[0] = results differing, out[1] =
 * the largest difference in ulps, out[2] = results differing by more than one
 * ulp.  The exact mode's square roots and quotients are correctly rounded (0
 * differing; its reciprocals and cube roots are the library's); the FMA mode's
 * are within an ulp. */
int fierro_root_check(int fp_mode, int which, long long n, unsigned long long seed, int lo_exp, int hi_exp,
                      unsigned long long* out);

/* Graphics dumps (write_outputs, outputs.cpp:10-506), written off the critical
 * path.  With outputs on, every write event of the cycle loop -- t = 0 of a
 * freshly uploaded state (sgh_solve.cpp:45) and each cycle that meets the write
 * condition (graphics_cyc_ival, graphics_time, time_final; sgh_solve.cpp:590-632)
 * -- snapshots the state into a device ring of `slots` slots; a writer thread
 * of the handle writes, under `directory`, the reference's files byte for byte:
 * FIERRO_OUTPUT_ENSIGHT  ensight/Outputs_SGH.case, ensight/data/Outputs_SGH.NNNNN.*
 * FIERRO_OUTPUT_STATE    state/elem_state_t<time>.txt
 * Snapshots are taken by fierro_sgh_run / fierro_sgh_enqueue_cycles (which then
 * keep at most two cycles in flight beyond the free slots), not by the stage-
 * stepping and event-timed entry points.  directory == NULL or what == 0 turns
 * outputs off.  A new set_state restarts the numbering at 00000. */
#define FIERRO_OUTPUT_ENSIGHT 1
#define FIERRO_OUTPUT_STATE 2
int fierro_sgh_set_output(fierro_sgh* h, const char* directory, int what, int slots);
/* Waits until every snapshot taken so far is written; *dumps = dumps written
 * since the last set_state.  Reports a write error of the writer thread. */
int fierro_sgh_flush_output(fierro_sgh* h, int64_t* dumps);

/* Device-resident state of a handle for zero-copy use (e.g. torch tensors over
 * the same memory).  Arrays are in the device numbering (Morton order); the
 * maps convert: caller id = *_int2ext[device id], device id = *_ext2int[caller
 * id].  Valid until the next call that runs cycles or uploads a state (the
 * state bins swap each cycle); work on them belongs on `stream` or after
 * fierro_sgh_synchronize.  No counterpart in the reference (its device mirror
 * is private to the DViewCArrayKokkos objects). */
typedef struct {
  int64_t num_nodes, num_elems;
  double *x, *y, *z, *u, *v, *w, *node_mass;                 /* [Nn] */
  double *den, *pres, *sspd, *sie, *vol, *mass, *div;        /* [Ne] */
  double* corner_force;                                      /* [24][Ne], row lid*3+dim */
  const int32_t *node_int2ext, *elem_int2ext, *node_ext2int, *elem_ext2int;
  void* stream;                                              /* the handle's cudaStream_t */
} fierro_device_view;
int fierro_sgh_device_view(fierro_sgh* h, fierro_device_view* view);

/* ---- discrete adjoint of the cycle loop ------------------------------------
 * No counterpart in the reference, which has no adjoint; these differentiate the
 * loop that fierro_sgh_run executes (sgh_solve.cpp:125-634), with the
 * parameters an element's initial specific internal energy and gamma
 * (elem_statev[e][0]).  The pair is shaped like a torch.autograd.Function:
 * forward runs the loop and keeps what backward needs; backward maps adjoints
 * of the final state to adjoints of the parameters.  Exact arithmetic mode and
 * handles without strength materials only (FIERRO_ENOTSUP otherwise).
 *
 * fierro_adj_forward: from the handle's current state (a cycle boundary, e.g.
 * right after set_state), replaces elem_sie (bin 1) by sie0[Ne] and gamma by
 * gamma[Ne] (either may be NULL: keep the current values), recomputes pressure
 * and sound speed from them with the ideal-gas EOS, then runs `cycles` cycles
 * exactly as fierro_sgh_run does, keeping a device-resident checkpoint every
 * ckpt_every cycles.  The final state is then read with fierro_sgh_get_state.
 * Device memory: checkpoints (6 Nn + 30 Ne doubles each) plus a replay tape of
 * ckpt_every cycles ((2 ckpt_every + 1)(9 Nn + 30 Ne) + 48 ckpt_every Ne doubles
 * for two RK stages); FIERRO_ENOMEM if it does not fit. */
int fierro_adj_forward(fierro_sgh* h, const double* sie0, const double* gamma, int64_t cycles,
                       int64_t ckpt_every, int64_t* cycles_run);

/* Adjoints of the final state (d J / d field), host arrays in the caller's
 * numbering; NULL fields are zero.  Element fields [Ne]; coords and vel
 * [Nn][3] (bin 1). */
typedef struct {
  const double* den;
  const double* pres;
  const double* sie;
  const double* sspd;
  const double* vol;
  const double* coords;
  const double* vel;
} fierro_adj_seed;

/* fierro_adj_backward: replays each checkpoint segment (bit-identical to the
 * forward) and runs the reverse pass.  Writes d J / d sie0 [Ne], d J / d gamma
 * [Ne] (per element; the derivative for one material-wide gamma is their sum)
 * and d J / d initial node velocity [Nn][3]; any output may be NULL.  Switches
 * of the forward (limiter, Mach switch, compression, CFL minimiser, dt clamps)
 * are differentiated on the side the forward took.  The state must be the one
 * fierro_adj_forward left; backward may be called repeatedly with other seeds. */
int fierro_adj_backward(fierro_sgh* h, const fierro_adj_seed* seed, double* sie0_bar, double* gamma_bar,
                        double* vel0_bar);

/* enable != 0: backward also recomputes every corner force of the replay inside
 * the reverse force kernel and fails (FIERRO_ENUMERIC) unless all match bit for
 * bit; a self-check of the reverse pass's forward values. */
int fierro_adj_verify(fierro_sgh* h, int enable);

/* out[0..n), n <= 11: cycles of the last forward, checkpoint interval,
 * segments, tape bytes, checkpoint bytes, total adjoint device bytes; of the last
 * backward: force mismatches, status bits, and the number of cycles whose dt came
 * from the CFL minimum, from the growth cap, and from the other clamps. */
int fierro_adj_stats(const fierro_sgh* h, int64_t* out, int64_t n);

/* Frees the adjoint's device memory (also done by fierro_sgh_destroy). */
int fierro_adj_release(fierro_sgh* h);

/* Frozen-branch forward (no counterpart in the reference).  The forward has
 * switches: the corner force's compression coefficients (div < 0), the Riemann
 * velocity's guard, the shock limiter's minimising neighbour and its clamps to
 * [0, 1], the Mach switch min(1, .) (force_sgh.cpp:147-329), and the time
 * step's CFL minimiser (element and node pair), growth cap and clamps
 * (time_integration.cpp:54-154).  J is therefore piecewise smooth, and the
 * adjoint is the derivative of the piece the forward's own run lies on.
 *   FIERRO_ADJ_BRANCHES_RECORD: the next fierro_adj_forward calls also record
 *     every such decision, cycle by cycle (1 + 4 bytes per element per RK stage
 *     per cycle, plus one record per cycle; the forward's values are unchanged);
 *   FIERRO_ADJ_BRANCHES_FREEZE: fierro_adj_forward runs with the decisions of
 *     the recorded run instead of making them (same cycle count; no checkpoints,
 *     and no fierro_adj_backward after it).  On the recorded parameters it
 *     reproduces the recorded run bit for bit; for other parameters its result
 *     is the smooth piece the adjoint differentiates, so its central
 *     differences check the adjoint without straddling the switches;
 *   FIERRO_ADJ_BRANCHES_OFF: plain forwards again; frees the record.
 * Exact-mode gas-only hex handles (FIERRO_ENOTSUP otherwise). */
#define FIERRO_ADJ_BRANCHES_OFF 0
#define FIERRO_ADJ_BRANCHES_RECORD 1
#define FIERRO_ADJ_BRANCHES_FREEZE 2
int fierro_adj_branches(fierro_sgh* h, int mode);

#ifdef __cplusplus
}
#endif
#endif /* FIERRO_SGH_H */
