// Device data layout and per-launch argument records of the SGH kernels.
//
// HBM layout (internal, Morton-ordered numbering):
//   nodes    SoA float64: x,y,z and u,v,w in two ping-pong bins (cycle-start and
//            current), half-velocity hx,hy,hz of the current stage, node mass,
//            boundary bit mask (uint8)
//   elements SoA float64: den, pres, sspd, vol, div, mass, gamma, c_min, sie in two
//            bins; int32 nodes_in_elem [ne][8]
//   bmat     [24][ne]  outward corner area normals B(lid, dim) of the current
//            geometry (row lid*3+dim), written by the element kernel and read by
//            the next stage's force kernel
//   force    [24][ne]  corner forces, row lid*3+dim
//   stress   two bins of [9][ne] (row i*3+j) and statev [nsv][ne], only on a
//            handle with a strength material
//   div      two buffers: the force pass of a stage reads one, the element pass
//            writes the next stage's into the other (so the reference-visible
//            elem_div, the one the last stage used, survives)
//   corner CSR per node (int32 corner id e*8+lid, reference summation order),
//   neighbour CSR per element (int32)
#ifndef FIERRO_SGH_DEVICE_H
#define FIERRO_SGH_DEVICE_H

#include <cstdint>

#include <cuda_runtime.h>

namespace fierro {

// Device-resident loop scalars (sgh_solve's time_value / dt / graphics_time).
struct Ctrl {
  double dt;
  double time_value;
  double graphics_time;
  long long cycle;     // completed cycles
  int active;          // the current cycle runs (set by the dt kernel)
  int stopped;         // time_value reached time_final
  unsigned int status; // FIERRO_STATUS_* bits
  int wrote;           // the last cycle ended with a write event (graphics dump)
};

#define FIERRO_STATUS_BAD_VOLUME 1u  // non-positive or non-finite element volume
#define FIERRO_STATUS_BAD_STATE 2u   // non-finite energy, pressure or velocity
#define FIERRO_STATUS_DT_FLOOR 4u    // a CFL step fell below dt_min and dt was raised to it (warning)

struct LoopParams {
  double time_final, dt_max, dt_min, dt_cfl, graphics_dt_ival, fuzz, small;
  long long graphics_cyc_ival;
};

struct ForceArgs {
  int ne;
  const int* nie;
  const int* eie_start;
  const int* eie;
  const int* mat;
  const double* qtab;  // [nmat][4] = q1, q1ex, q2, q2ex
  const double* bmat;
  const double *u, *v, *w;  // current velocity (reference bin 1)
  const double *den, *pres, *sspd, *vol;
  const double* div;  // divergence of this stage (written by the previous element pass)
  double* force;
  const Ctrl* ctrl;   // plain: the solver's control block; batch: one per instance
  const int* inst;    // batch only: instance of each element (negative = padding)
  double fuzz, small;
  // adjoint replay only (force_tape launcher): the viscosity intermediates of
  // each element, rows of kForceTapeRows x ne, and the limiter's neighbour
  double* tape;
  int* tape_sel;
  // adjoint branch record / freeze only (force_branch launcher): one byte of
  // branch bits per element (FIERRO_BR_* below) and the limiter's neighbour
  unsigned char* br_flags;
  int* br_sel;
  // strength materials (set when the handle has one; stress rows [9][ne],
  // row i*3+j): the reference's stress(1) as this stage's force reads it, the
  // cycle-start stress(0), and where the stage's stress(1) goes
  const double* stress_cur;
  const double* stress0;
  double* stress_out;
  const int* stype;    // [nmat] strength_type: 0 none, 1 hypo, 2 hyper
  double* statev;      // [nsv][ne] element state variables
  const double* sie0;  // cycle-start energy (the reference passes elem_sie bin 0)
  double rk_alpha;
  int copy_stress;     // stage 0: elements without a hypo model carry stress_cur over
  int block;           // threads per block (0: kForceBlock)
  int grid;            // batch only: blocks of a persistent grid (0: one block per tile)
};

// Branch bits of one element's corner force in one stage, recorded on a base
// trajectory and replayed by the frozen-branch forward (the forward whose
// central differences are the derivative the discrete adjoint computes).
#define FIERRO_BR_COMPRESS 1u   // div < 0: the compression coefficients q1, q2
#define FIERRO_BR_VSTAR 2u      // sum mu > fuzz: the Riemann velocity is the mu-weighted mean
#define FIERRO_BR_MACH_CLAMP 4u // the Mach switch's argument reached 1 (alpha = 1)
#define FIERRO_BR_LIM_SHIFT 3   // limiter case, 2 bits: FIERRO_LIM_*
#define FIERRO_LIM_NONE 0u      // r_min = 1 (no neighbour below): phi0 = 0
#define FIERRO_LIM_FACE 1u      // 0 < r_min < 1 at the recorded neighbour: phi0 = 1 - r_face
#define FIERRO_LIM_FULL 2u      // r_min <= 0: phi0 = 1
#define FIERRO_LIM_IRREGULAR 3u // non-finite or zero divergence: evaluated as the cycle does

// Rows of the force kernel's tape: mu[8], |v_l - v_avg|[8], v*[3], sum mu,
// phi0 (limiter), the Mach-switch argument, vol^(1/3), the limiter's r_min.
constexpr int kForceTapeRows = 24;

struct NodeArgs {
  int nn, ne;
  const int* cin_start;
  const int* cin;
  const double* force;
  const double* node_mass;
  const double* node_rm;  // 1 / node_mass, computed once per uploaded state (FMA mode; NULL: divide)
  const unsigned char* bc_mask;
  const double *u0, *v0, *w0, *x0, *y0, *z0;  // cycle start (reference bin 0)
  double *u1, *v1, *w1, *x1, *y1, *z1;        // updated (reference bin 1)
  double *hx, *hy, *hz;                       // half velocity (v1 + v0) / 2
  const Ctrl* ctrl;
  const int* inst;  // batch only: instance of each node
  double rk_alpha;
  int block;        // threads per block (0: kNodeBlock)
  int grid;         // batch only: blocks of a persistent grid (0: one block per node tile)
};

// kind: 0 = stage update, 1 = last stage of a cycle (adds the CFL partial
// minima), 2 = prime (geometry, divergence and CFL of the uploaded state only).
struct ElemArgs {
  int ne;
  const int* nie;
  const double *x, *y, *z;     // updated coordinates (reference bin 1)
  const double *u, *v, *w;     // updated velocity
  const double *hx, *hy, *hz;  // half velocity of this stage
  const double* force;
  const double* mass;
  const double* sie0;
  double* sie1;
  const double *gamma, *csmin;
  double *den, *pres, *sspd, *vol;
  double* div;  // divergence for the next stage
  double* bmat;
  long long* cfl_part;  // per-block minimum of the element time steps (order keys)
  Ctrl* ctrl;
  const int* inst;            // batch only: instance of each element (negative = padding)
  const double* dt_cfl_tab;   // batch only: CFL number per instance
  double rk_alpha, dt_cfl, fuzz;
  // hyper strength materials (set when the handle has one): stress rows [9][ne]
  const int* mat;
  const int* stype;
  const double* stress0;  // cycle-start stress(0)
  double* stress1;        // stress(1), updated in place
  double* statev;         // [nsv][ne]
  int block;              // threads per block, one CFL partial per tile of that many elements (0: kElemBlock;
                          // a batch's block divides kElemBlock)
  int grid;               // batch only: blocks of a persistent grid looping over the tiles (0: one per tile)
};

// Grid barrier of the batch's fused stage kernel: an arrival counter and a
// generation counter in device memory, and a status word a block sets when its
// wait ran out (the launch is cooperative, so every block is resident and the
// limit is only a guard).
struct StageSync {
  unsigned int* arrive;
  unsigned int* gen;
  unsigned int* status;
};
#define FIERRO_SYNC_TIMEOUT 1u

struct DtArgs {
  const long long* cfl_part;
  int nparts;
  Ctrl* ctrl;
  LoopParams lp;
  // batch only: instance i owns cfl_part[part_start[i] .. part_start[i+1])
  const int* part_start;
  const LoopParams* lps;
  int ninst;
};

struct EnergyArgs {
  int ne, nn;
  const double *mass, *sie;
  const double *node_mass, *u, *v, *w;
  double* part;  // [2][nblocks]
  double* out;   // [2]
};

// One arithmetic mode's launchers (defined in sgh_kernels.cu, compiled once per mode).
struct KernelSet {
  void (*force)(const ForceArgs&, cudaStream_t);
  void (*force_tape)(const ForceArgs&, cudaStream_t);  // the same, also writing a.tape / a.tape_sel
  // mode 1: the plain force, also recording a.br_flags / a.br_sel; mode 2: the
  // force with those branches frozen (gas-only hex handles, exact mode)
  void (*force_branch)(const ForceArgs&, int mode, cudaStream_t);
  void (*node)(const NodeArgs&, cudaStream_t);
  void (*elem)(const ElemArgs&, int kind, cudaStream_t);
  void (*dt)(const DtArgs&, cudaStream_t);
  void (*end)(Ctrl*, const LoopParams&, cudaStream_t);
  void (*energy)(const EnergyArgs&, cudaStream_t);
  void (*end_batch)(Ctrl*, const LoopParams*, int, cudaStream_t);
  const char* name;
  // resident blocks per SM of a batch kernel (0 force, 1 node, 2 element) at
  // `block` threads per block: the unit of a persistent grid
  int (*batch_max_blocks)(int kernel, int block);
  // out[i] = 1 / in[i] (IEEE division), i < n
  void (*reciprocal)(const double* in, double* out, int n, cudaStream_t);
  // the mode's square root, cube root, quotient or reciprocal (which 0..3)
  // against the library's on n seeded inputs: out[0] differing, out[1] largest
  // difference in ulps, out[2] differing by more than one ulp (fierro_root_check)
  void (*root_check)(int which, long long n, unsigned long long seed, int lo_exp, int hi_exp,
                     unsigned long long* out, cudaStream_t);
  // a batch's RK stage as one cooperative launch: the force, node and element
  // passes over `grid` resident blocks of ea.block threads with grid barriers
  // between them (kind as for elem; cooperative 0 only for the timeout test);
  // and that kernel's resident blocks per SM
  cudaError_t (*stage_fused)(const ForceArgs& fa, const NodeArgs& na, const ElemArgs& ea, int kind,
                             const StageSync& sync, int grid, int cooperative, cudaStream_t);
  int (*fused_max_blocks)(int block);
};

constexpr int kElemBlock = 128;
constexpr int kForceBlock = 128;
constexpr int kNodeBlock = 256;
constexpr int kEnergyBlock = 256;

// Launch block for `n` threads of a kernel whose default block is `bs`: halved
// (down to one warp) while the grid would have fewer than kMinBlocks blocks, so a
// small mesh spreads over more SMs (each SM's FP64 rate, not the chip's, bounds
// a kernel that occupies few of them).  It depends on n alone, so the number of
// CFL partials (one per element block) is a property of the mesh.
constexpr long long kMinBlocks = 304;  // two per SM of a 152-SM GB300
inline int small_mesh_block(long long n, int bs) {
  while (bs > 32 && (n + bs - 1) / bs < kMinBlocks) bs >>= 1;
  return bs;
}

const KernelSet& kernels_exact();
const KernelSet& kernels_fma();

}  // namespace fierro

#endif
