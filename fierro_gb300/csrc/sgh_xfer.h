// Direct host<->device state transfer (sgh_xfer.cu): the GPU reads and writes the
// caller's host arrays itself where the device can dereference pageable host
// memory (GB300: address translation over NVLink-C2C).
#ifndef FIERRO_SGH_XFER_H
#define FIERRO_SGH_XFER_H

#include "fierro_sgh.h"
#include "sgh_device.h"

struct fierro_sgh;

namespace fierro {

// Validation result of an upload: bit k of `flags` set when check k failed,
// first[k] = the smallest caller index (element, node or stress value) that
// failed it.
struct XferStatus {
  enum { STRESS = 0, MAT_ID = 1, VOLUME = 2, MASS = 3, NODE_MASS = 4, COUNT = 5 };
  unsigned int flags;
  int pad;
  long long first[COUNT];
};

namespace xfer {

// True when kernels may dereference pageable host pointers on the current device.
bool direct_host_access();
// Uploads a state (reference layouts) into the handle's bins and reports the
// validation result; the state on the device is the caller's even when a check
// failed (the caller then discards it).  A strength handle also takes the stress
// bins and all num_state_vars state variables (h->d_statev sized for them).
// With wait == false the transfers are only enqueued on the handle's stream and
// `status` is not written: the caller does host work meanwhile, then calls
// finish_upload.
int upload_state(fierro_sgh* h, const fierro_sgh_state* s, XferStatus* status, bool wait = true);
int finish_upload(fierro_sgh* h, XferStatus* status);
// Writes the handle's state into the non-null fields of `s`: reference bin rb
// from device bin bins[rb]; elem_div from divergence buffer div_buffer.  On a
// handle with strength materials the stress bins and the state variables come
// from the device; otherwise the stress is zero and elem_statev is not written.
// wait == false: enqueued only; the caller synchronises the handle's stream.
int download_state(fierro_sgh* h, fierro_sgh_state* s, const int bins[2], int div_buffer, bool wait = true);

// Graphics-dump snapshots (write_outputs, outputs.cpp:10-506): one slot of the
// device ring holds, in the caller's numbering, node rows x, y, z, u, v, w
// (kSnapNodeRows x nn) then element rows den, pres, sie, vol, mass, sspd,
// speed, mat_id, centroid x, y, z, radius_2D, radius_3D (kSnapElemRows x ne).
constexpr int kSnapNodeRows = 6, kSnapElemRows = 13;

struct SnapArgs {
  int nn, ne, nslots, force;  // force: snapshot whether or not the cycle wrote
  const Ctrl* ctrl;
  const int *node_ext2int, *elem_ext2int, *nie;  // nie: internal [ne][8]
  const double *x, *y, *z, *u, *v, *w;           // the state bin after the cycle
  const double *den, *pres, *sie, *vol, *mass, *sspd;
  const int* mat;
  double* ring;                  // nslots slots
  double* times;                 // [nslots] time_value of each slot
  unsigned long long* count;     // snapshots taken (device)
  unsigned long long* produced;  // host-mapped mirror of count, written last
};

// Two launches on `s`: the gather (a no-op unless ctrl->wrote or force) and the
// single-thread publication of the slot's time and the new count.
void launch_snapshot(const SnapArgs& a, cudaStream_t s);

}  // namespace xfer
}  // namespace fierro

#endif
