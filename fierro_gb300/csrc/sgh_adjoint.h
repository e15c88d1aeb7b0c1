// Discrete adjoint of the SGH cycle: device data layout and launcher records.
//
// Tape (one checkpoint segment of k cycles, S RK stages each):
//   Slot j = 0 .. k*S    the state at stage boundary j (slot 0 = checkpoint), one
//                        contiguous block: node x,y,z,u,v,w,hx,hy,hz [9][nn], then
//                        element sie,vol,den,pres,sspd,div [6][ne], bmat [24][ne]
//   force j = 0 .. k*S-1 corner forces of stage j [24][ne], and the force kernel's
//                        viscosity intermediates [kForceTapeRows][ne] + limiter
//                        neighbour [ne] (the reverse force pass reads them)
//   AdjRecord per cycle  the dt computation's inputs and result
// Checkpoint g: node x..w [6][nn], element sie..div + bmat [30][ne], Ctrl and the
// CFL block minima, i.e. exactly slot 0 of segment g plus the loop scalars.
//
// Adjoint buffers ("bar" = adjoint, d J / d value):
//   bbar, volbar, divbar, nbv/nbc   adjoints of the derived fields (corner normals,
//                                   volume, divergence) of the state being
//                                   reversed into; nbv/nbc carry the limiter's
//                                   neighbour-divergence term to that neighbour
//   cx, cv [24][ne]                 per-corner contributions to node coordinate /
//                                   velocity adjoints, summed per node by the node
//                                   reverse kernel (no atomics, fixed order)
//   w [ne]                          adjoint of the element power (-adt/M * siebar)
//   fbar [3][nn]                    adjoint of the summed node force
//   sb[2], sbt [ne]                 sie adjoints: cycle start (two, swapped per
//                                   cycle) and an intermediate stage
//   an[2][6][nn]                    direct adjoints of cycle-start x,y,z,u,v,w
//   gbar [ne]                       gamma adjoint (summed over the whole run)
#ifndef FIERRO_SGH_ADJOINT_H
#define FIERRO_SGH_ADJOINT_H

#include "sgh_device.h"

namespace fierro {

struct Slot {
  double *x, *y, *z, *u, *v, *w;
  double *hx, *hy, *hz;
  double *sie, *vol, *den, *pres, *sspd, *div;
  double* bmat;
};

// One cycle's time-step computation (time_integration.cpp:54-154, sgh_solve.cpp:590-632).
struct AdjRecord {
  double dt_prev, time_value, graphics_time, dt;  // before the cycle; dt chosen by it
  long long cfl_key;                              // order key of the CFL minimum
  long long cycle;                                // completed cycles before it
  int estar;                                      // element attaining the CFL minimum
  int active;
  int pair;                                       // its node pair attaining the minimum (branch record)
};

#define FIERRO_ADJ_STATUS_DT_MISMATCH 1u  // re-derived dt differs from the recorded one

struct AdjScalars {
  double dt_carry;   // adjoint of the previous cycle's dt through the growth cap
  double time_bar;   // adjoint of time_value
  double gtime_bar;  // adjoint of graphics_time
  unsigned int status;
  int n_cfl;         // reversed cycles whose dt came from the CFL minimum
  int n_grow;        // ... from the growth cap
  int n_other;       // ... from dt_min/dt_max or the graphics/final-time clamps
};

struct AdjMesh {
  int ne, nn;
  const int *nie, *eie_start, *eie, *cin_start, *cin, *mat;
  const double* qtab;
  const unsigned char* bc;
  const double *elem_mass, *node_mass, *gamma, *csmin;
};

struct AdjBufs {
  double* bbar;
  double *volbar, *divbar, *nbv;
  int* nbc;
  double *cx, *cv;
  double* w;
  double* fbar[3];
  double* gbar;
  double* sbt;
  double *part_e, *part_n;  // [S][blocks] adjoint of rk_alpha*dt per stage
  int nbe, nbn;
  AdjScalars* sc;
  unsigned long long* mismatch;  // optional: count of recomputed forces that differ
};

struct AdjAlphas {
  double a[8];
};

// Six node arrays (x, y, z, u, v, w), passed by value; a null entry reads as zero.
struct Node6 {
  double* p[6];
};

struct AdjLaunch {
  void (*eos)(int ne, const double* sie, const double* den, const double* gamma, const double* csmin,
              double* pres, double* sspd, cudaStream_t);
  void (*pre)(AdjRecord* r, const long long* cfl_part, int nparts, const Ctrl* ctrl, cudaStream_t);
  void (*argmin)(AdjRecord* r, const Ctrl* ctrl, const LoopParams& lp, const AdjMesh& m, const Slot& s,
                 cudaStream_t);
  // eseed [5][ne] (den, pres, sie, sspd, vol), nseed [6][nn] (x, y, z, u, v, w);
  // bit i of seed_mask marks seed i present (elements 0..4, nodes 5..10)
  void (*seed)(const AdjMesh& m, const AdjBufs& b, const Slot& fin, const double* eseed, const double* nseed,
               unsigned seed_mask, double* sb_next, const Node6& an_next, cudaStream_t);
  // kind 0: stage; 2: the uploaded (primed) state
  void (*elem)(const AdjMesh& m, const AdjBufs& b, const Slot& s1, const double* force, const AdjRecord* r,
               double alpha, const double* sie_in, double* sie_c, int assign, double* part, int kind,
               cudaStream_t);
  void (*node)(const AdjMesh& m, const AdjBufs& b, const Slot& s1, const double* force, const AdjRecord* r,
               double alpha, const Node6& an_in, const Node6& an_c, int assign, double* part, cudaStream_t);
  // ft / fsel: the replay's force tape of this stage (kForceTapeRows x ne, ne)
  void (*force)(const AdjMesh& m, const AdjBufs& b, const Slot& s0, const Slot& s1, const double* force_tape,
                const double* ft, const int* fsel, double fuzz, double small, double* sie_out, int accumulate,
                cudaStream_t);
  void (*dt)(const AdjMesh& m, const AdjBufs& b, const AdjRecord* r, const LoopParams& lp, const Slot& s0,
             int stages, const AdjAlphas& al, const Node6& an_c, double* sie_c, cudaStream_t);
  // velocity adjoint of the uploaded state into b.fbar[0..2]
  void (*vel0)(const AdjMesh& m, const AdjBufs& b, const Node6& an, cudaStream_t);
  // branch record: the node pair of the recorded CFL element (after argmin)
  void (*pair)(AdjRecord* r, const AdjMesh& m, const Slot& s, cudaStream_t);
  // frozen-branch forward: the cycle's dt along the recorded dt branch, from
  // the current state s and loop scalars
  void (*dt_frozen)(const AdjRecord* r, Ctrl* ctrl, const LoopParams& lp, const AdjMesh& m, const Slot& s,
                    cudaStream_t);
};

const AdjLaunch& adjoint_kernels();

}  // namespace fierro

#endif
