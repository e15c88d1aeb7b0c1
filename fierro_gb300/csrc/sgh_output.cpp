// Graphics dumps off the critical path: write_outputs (outputs.cpp:10-506) for a
// handle.  A write event of the cycle loop (sgh_solve.cpp:45 at t = 0 and
// :590-632 afterwards) makes the cycle graph gather the state into a slot of a
// device-resident ring (sgh_xfer.cu); a host writer thread copies finished slots
// out on its own stream and writes the reference's files -- EnSight Gold
// (ensight/Outputs_SGH.case, ensight/data/Outputs_SGH.NNNNN.{geo,den,...}) and
// the element state text (state/elem_state_t<time>.txt) -- byte for byte in the
// reference's formats, formatting in parallel.  The GPU never waits for the
// files unless the ring is full: fierro_sgh_run keeps at most two cycles in
// flight beyond what the free slots can absorb.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <deque>
#include <string>
#include <thread>
#include <vector>

#include <sys/stat.h>

#include "sgh_handle.h"

using namespace fierro;
using namespace fierro::hd;

namespace fierro {

struct OutputState {
  std::string dir;
  int what = 0;
  int nslots = 0;
  size_t slot_doubles = 0;
  double* d_ring = nullptr;
  double* d_times = nullptr;
  unsigned long long* d_count = nullptr;
  unsigned long long* h_produced = nullptr;  // mapped pinned
  unsigned long long* d_produced = nullptr;
  std::atomic<unsigned long long> consumed{0};
  std::atomic<bool> stop{false};
  std::thread writer;
  cudaStream_t copy_stream = nullptr;
  double* h_slot = nullptr;  // pinned, one slot
  std::vector<double> times;
  std::string conn_text, switch_text;
  std::atomic<int> error{0};
  std::string error_msg;
  bool t0_pending = true;
  std::deque<cudaEvent_t> in_flight;  // end events of enqueued cycles
  std::vector<cudaEvent_t> event_pool;
  long long nn = 0, ne = 0;
};

}  // namespace fierro

namespace {

const char* kName = "Outputs_SGH";
const char* kScalarNames[9] = {"den", "pres", "sie", "vol", "mass", "sspd", "speed", "mat_id", "elem_switch"};
const char* kVecNames[2] = {"pos", "vel"};

void mkdir_p(const std::string& d) { ::mkdir(d.c_str(), 0755); }

// printf-formatted values, formatted in parallel chunks and written in order.
bool write_values(FILE* f, const double* v, size_t n, const char* fmt) {
  const size_t chunk = 1 << 15;
  const int64_t nc = (int64_t)((n + chunk - 1) / chunk);
  std::vector<std::string> bufs((size_t)nc);
#pragma omp parallel for schedule(dynamic)
  for (int64_t c = 0; c < nc; ++c) {
    std::string& s = bufs[(size_t)c];
    const size_t lo = (size_t)c * chunk, hi = std::min(n, lo + chunk);
    s.reserve((hi - lo) * 14);
    char tmp[64];
    for (size_t i = lo; i < hi; ++i) {
      const int k = std::snprintf(tmp, sizeof(tmp), fmt, v[i]);
      s.append(tmp, (size_t)k);
    }
  }
  for (auto& s : bufs)
    if (std::fwrite(s.data(), 1, s.size(), f) != s.size()) return false;
  return true;
}

FILE* open_or_fail(OutputState* o, const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f && !o->error.load()) {
    o->error_msg = "cannot open " + path;
    o->error.store(FIERRO_EINVAL);
  }
  return f;
}

void write_dump(OutputState* o, const double* slot, double time_value) {
  const size_t nn = (size_t)o->nn, ne = (size_t)o->ne;
  const double* nodes = slot;
  const double* el = slot + xfer::kSnapNodeRows * nn;
  const size_t gid = o->times.size();
  o->times.push_back(time_value);
  char name[512];
  if (o->what & FIERRO_OUTPUT_STATE) {
    // state_file (outputs.cpp:413-506)
    mkdir_p(o->dir + "/state");
    std::snprintf(name, sizeof(name), "%s/state/elem_state_t%6.5e.txt", o->dir.c_str(), time_value);
    if (FILE* f = open_or_fail(o, name)) {
      std::fputs("# state dump file\n", f);
      std::fputs("# x  y  z  radius_2D  radius_3D  den  pres  sie  sspd  vol  mass \n", f);
      const size_t chunk = 1 << 14;
      const int64_t nc = (int64_t)((ne + chunk - 1) / chunk);
      std::vector<std::string> bufs((size_t)nc);
#pragma omp parallel for schedule(dynamic)
      for (int64_t c = 0; c < nc; ++c) {
        std::string& s = bufs[(size_t)c];
        char tmp[512];
        for (size_t E = (size_t)c * chunk; E < std::min(ne, (size_t)(c + 1) * chunk); ++E) {
          const int k = std::snprintf(tmp, sizeof(tmp),
                                      "%f\t %f\t %f\t %f\t %f\t %f\t %f\t %f\t %f\t %f\t %f\t \n",
                                      el[8 * ne + E], el[9 * ne + E], el[10 * ne + E], el[11 * ne + E],
                                      el[12 * ne + E], el[E], el[ne + E], el[2 * ne + E], el[5 * ne + E],
                                      el[3 * ne + E], el[4 * ne + E]);
          s.append(tmp, (size_t)k);
        }
      }
      for (auto& s : bufs) std::fwrite(s.data(), 1, s.size(), f);
      std::fclose(f);
    }
  }
  if (o->what & FIERRO_OUTPUT_ENSIGHT) {
    // ensight (outputs.cpp:85-409)
    mkdir_p(o->dir + "/ensight");
    mkdir_p(o->dir + "/ensight/data");
    std::snprintf(name, sizeof(name), "%s/ensight/data/%s.%05lu.geo", o->dir.c_str(), kName, (unsigned long)gid);
    if (FILE* f = open_or_fail(o, name)) {
      std::fputs("A graphics dump by Fierro \n", f);
      std::fputs("EnSight Gold geometry\n", f);
      std::fputs("node id assign\n", f);
      std::fputs("element id assign\n", f);
      std::fputs("part\n", f);
      std::fprintf(f, "%10d\n", 1);
      std::fputs("Mesh\n", f);
      std::fputs("coordinates\n", f);
      std::fprintf(f, "%10lu\n", (unsigned long)nn);
      write_values(f, nodes, 3 * nn, "%12.5e\n");
      std::fputs("hexa8\n", f);
      std::fprintf(f, "%10lu\n", (unsigned long)ne);
      std::fwrite(o->conn_text.data(), 1, o->conn_text.size(), f);
      std::fclose(f);
    }
    for (int var = 0; var < 9; ++var) {
      std::snprintf(name, sizeof(name), "%s/ensight/data/%s.%05lu.%s", o->dir.c_str(), kName, (unsigned long)gid,
                    kScalarNames[var]);
      FILE* f = open_or_fail(o, name);
      if (!f) continue;
      std::fputs("Per_elem scalar values\n", f);
      std::fputs("part\n", f);
      std::fprintf(f, "%10d\n", 1);
      std::fputs("hexa8\n", f);
      if (var < 8) write_values(f, el + (size_t)var * ne, ne, "%12.5e\n");
      else std::fwrite(o->switch_text.data(), 1, o->switch_text.size(), f);
      std::fclose(f);
    }
    for (int var = 0; var < 2; ++var) {
      std::snprintf(name, sizeof(name), "%s/ensight/data/%s.%05lu.%s", o->dir.c_str(), kName, (unsigned long)gid,
                    kVecNames[var]);
      FILE* f = open_or_fail(o, name);
      if (!f) continue;
      std::fputs("Per_node vector values\n", f);
      std::fputs("part\n", f);
      std::fprintf(f, "%10d\n", 1);
      std::fputs("block\n", f);
      write_values(f, nodes + (size_t)var * 3 * nn, 3 * nn, "%12.5e\n");
      std::fclose(f);
    }
    std::snprintf(name, sizeof(name), "%s/ensight/%s.case", o->dir.c_str(), kName);
    if (FILE* f = open_or_fail(o, name)) {
      std::fputs("FORMAT\n", f);
      std::fputs("type: ensight gold\n", f);
      std::fputs("GEOMETRY\n", f);
      std::fprintf(f, "model: data/%s.*****.geo\n", kName);
      std::fputs("VARIABLE\n", f);
      for (int var = 0; var < 9; ++var)
        std::fprintf(f, "scalar per element: %s data/%s.*****.%s\n", kScalarNames[var], kName, kScalarNames[var]);
      for (int var = 0; var < 2; ++var)
        std::fprintf(f, "vector per node: %s data/%s.*****.%s\n", kVecNames[var], kName, kVecNames[var]);
      std::fputs("TIME\n", f);
      std::fputs("time set: 1\n", f);
      std::fprintf(f, "number of steps: %4lu\n", (unsigned long)(gid + 1));
      std::fputs("filename start number: 0\n", f);
      std::fputs("filename increment: 1\n", f);
      std::fputs("time values: \n", f);
      for (double t : o->times) std::fprintf(f, "%12.5e\n", t);
      std::fclose(f);
    }
  }
}

void writer_loop(OutputState* o) {
  const size_t bytes = sizeof(double) * o->slot_doubles;
  for (;;) {
    const unsigned long long prod = *(volatile unsigned long long*)o->h_produced;
    const unsigned long long cons = o->consumed.load();
    if (cons < prod) {
      const size_t slot = (size_t)(cons % (unsigned long long)o->nslots);
      double t = 0.0;
      cudaError_t e1 = cudaMemcpyAsync(o->h_slot, o->d_ring + slot * o->slot_doubles, bytes, cudaMemcpyDeviceToHost,
                                       o->copy_stream);
      cudaError_t e2 = cudaMemcpyAsync(&t, o->d_times + slot, sizeof(double), cudaMemcpyDeviceToHost, o->copy_stream);
      cudaError_t e3 = cudaStreamSynchronize(o->copy_stream);
      if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) {
        if (!o->error.load()) {
          o->error_msg = std::string("snapshot copy: ") + cudaGetErrorString(e3 != cudaSuccess ? e3 : e1);
          o->error.store(FIERRO_ECUDA);
        }
      } else {
        write_dump(o, o->h_slot, t);
      }
      o->consumed.store(cons + 1);
      continue;
    }
    if (o->stop.load()) break;
    std::this_thread::sleep_for(std::chrono::microseconds(200));
  }
}

}  // namespace

namespace fierro {

void output_release(fierro_sgh* h) {
  OutputState* o = h ? h->out : nullptr;
  if (!o) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  o->stop.store(true);
  if (o->writer.joinable()) o->writer.join();
  for (cudaEvent_t e : o->event_pool) cudaEventDestroy(e);
  for (cudaEvent_t e : o->in_flight) cudaEventDestroy(e);
  if (o->copy_stream) cudaStreamDestroy(o->copy_stream);
  if (o->h_slot) cudaFreeHost(o->h_slot);
  if (o->h_produced) cudaFreeHost(o->h_produced);
  cudaFree(o->d_ring);
  cudaFree(o->d_times);
  cudaFree(o->d_count);
  delete o;
  h->out = nullptr;
}

xfer::SnapArgs output_snap_args(fierro_sgh* h, int bin, int force) {
  OutputState* o = h->out;
  xfer::SnapArgs a{};
  a.nn = (int)h->nn;
  a.ne = (int)h->ne;
  a.nslots = o->nslots;
  a.force = force;
  a.ctrl = h->d_ctrl;
  a.node_ext2int = h->d_node_ext2int;
  a.elem_ext2int = h->d_elem_ext2int;
  a.nie = h->d_nie;
  a.x = h->d_x[bin][0];
  a.y = h->d_x[bin][1];
  a.z = h->d_x[bin][2];
  a.u = h->d_v[bin][0];
  a.v = h->d_v[bin][1];
  a.w = h->d_v[bin][2];
  a.den = h->d_den;
  a.pres = h->d_pres;
  a.sie = h->d_sie[bin];
  a.vol = h->d_vol;
  a.mass = h->d_elem_mass;
  a.sspd = h->d_sspd;
  a.mat = h->d_mat;
  a.ring = o->d_ring;
  a.times = o->d_times;
  a.count = o->d_count;
  a.produced = o->d_produced;
  return a;
}

// Before enqueueing one cycle: the t = 0 dump of a fresh state, then wait until
// the ring can absorb the snapshots of every cycle in flight plus this one.
int output_before_cycle(fierro_sgh* h, long long cycles_done) {
  OutputState* o = h->out;
  if (!o) return FIERRO_OK;
  if (o->t0_pending && cycles_done == 0) {
    while ((long long)(*(volatile unsigned long long*)o->h_produced - o->consumed.load()) >= o->nslots)
      std::this_thread::sleep_for(std::chrono::microseconds(100));
    xfer::launch_snapshot(output_snap_args(h, bin_now(h, 0), 1), h->stream);
    CUDA_TRY(cudaGetLastError());
  }
  o->t0_pending = false;
  for (;;) {
    while (!o->in_flight.empty() && cudaEventQuery(o->in_flight.front()) == cudaSuccess) {
      o->event_pool.push_back(o->in_flight.front());
      o->in_flight.pop_front();
    }
    if (o->in_flight.size() >= 2) {
      CUDA_TRY(cudaEventSynchronize(o->in_flight.front()));
      continue;
    }
    // in flight: the t = 0 snapshot (if not yet published) is counted by
    // `produced` once it lands; every enqueued cycle may add one
    const unsigned long long prod = *(volatile unsigned long long*)o->h_produced;
    const long long pending = (long long)(prod - o->consumed.load()) + (long long)o->in_flight.size() + 1 + 1;
    if (pending <= o->nslots) break;
    if (o->error.load()) break;
    std::this_thread::sleep_for(std::chrono::microseconds(100));
  }
  return FIERRO_OK;
}

int output_after_cycle(fierro_sgh* h) {
  OutputState* o = h->out;
  if (!o) return FIERRO_OK;
  cudaEvent_t e = nullptr;
  if (!o->event_pool.empty()) {
    e = o->event_pool.back();
    o->event_pool.pop_back();
  } else {
    CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  CUDA_TRY(cudaEventRecord(e, h->stream));
  o->in_flight.push_back(e);
  return FIERRO_OK;
}

void output_reset(fierro_sgh* h) {
  OutputState* o = h->out;
  if (!o) return;
  // a new state starts a new series: wait for the old one, restart numbering
  if (h->stream) cudaStreamSynchronize(h->stream);
  while (o->consumed.load() < *(volatile unsigned long long*)o->h_produced)
    std::this_thread::sleep_for(std::chrono::microseconds(200));
  o->times.clear();
  o->t0_pending = true;
}

}  // namespace fierro

extern "C" int fierro_sgh_flush_output(fierro_sgh* h, int64_t* dumps) {
  clear_error();
  if (!h) return set_error(FIERRO_EINVAL, "handle is NULL");
  OutputState* o = h->out;
  if (dumps) *dumps = 0;
  if (!o) return FIERRO_OK;
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  while (o->consumed.load() < *(volatile unsigned long long*)o->h_produced)
    std::this_thread::sleep_for(std::chrono::microseconds(200));
  if (dumps) *dumps = (int64_t)o->times.size();
  if (o->error.load()) return set_error(o->error.load(), "output: %s", o->error_msg.c_str());
  return FIERRO_OK;
}

extern "C" int fierro_sgh_set_output(fierro_sgh* h, const char* directory, int what, int slots) {
  clear_error();
  if (!h) return set_error(FIERRO_EINVAL, "handle is NULL");
  output_release(h);
  if (!directory || what == 0) return fierro::rebuild_graphs(h);
  if (h->dims == 2) return set_error(FIERRO_ENOTSUP, "set_output: graphics dumps of hex meshes only");
  if ((what & ~(FIERRO_OUTPUT_ENSIGHT | FIERRO_OUTPUT_STATE)) != 0 || slots < 2 || slots > 1024)
    return set_error(FIERRO_EINVAL, "set_output: unknown output kinds or slots outside 2..1024");
  OutputState* o = new (std::nothrow) OutputState();
  if (!o) return set_error(FIERRO_ENOMEM, "host allocation failed");
  h->out = o;
  o->dir = directory;
  o->what = what;
  o->nslots = slots;
  o->nn = h->nn;
  o->ne = h->ne;
  o->slot_doubles = (size_t)xfer::kSnapNodeRows * (size_t)h->nn + (size_t)xfer::kSnapElemRows * (size_t)h->ne;
  auto fail = [&](int rc) {
    std::string msg = fierro_last_error();
    output_release(h);
    return set_error(rc, "%s", msg.c_str());
  };
  mkdir_p(o->dir);
  struct stat st;
  if (::stat(o->dir.c_str(), &st) != 0 || !S_ISDIR(st.st_mode))
    return fail(set_error(FIERRO_EINVAL, "set_output: %s is not a directory", directory));
  cudaError_t err = cudaMalloc(&o->d_ring, sizeof(double) * o->slot_doubles * (size_t)slots);
  if (err == cudaSuccess) err = cudaMalloc(&o->d_times, sizeof(double) * (size_t)slots);
  if (err == cudaSuccess) err = cudaMalloc(&o->d_count, sizeof(unsigned long long));
  if (err == cudaSuccess) err = cudaHostAlloc((void**)&o->h_produced, sizeof(unsigned long long), cudaHostAllocMapped);
  if (err == cudaSuccess) err = cudaHostGetDevicePointer((void**)&o->d_produced, o->h_produced, 0);
  if (err == cudaSuccess) err = cudaHostAlloc((void**)&o->h_slot, sizeof(double) * o->slot_doubles, cudaHostAllocDefault);
  if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&o->copy_stream, cudaStreamNonBlocking);
  if (err != cudaSuccess) return fail(set_error(FIERRO_ENOMEM, "set_output: %s", cudaGetErrorString(err)));
  *o->h_produced = 0;
  if (cudaMemsetAsync(o->d_count, 0, sizeof(unsigned long long), h->stream) != cudaSuccess)
    return fail(set_error(FIERRO_ECUDA, "set_output: memset"));
  // the connectivity text of the geometry file, caller numbering, 1-based
  {
    const size_t ne = (size_t)h->ne;
    std::vector<int32_t> nie(ne * 8);
    if (cudaMemcpy(nie.data(), h->d_nie, sizeof(int32_t) * ne * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
      return fail(set_error(FIERRO_ECUDA, "set_output: connectivity download"));
    const HostTopo& t = h->topo;
    std::vector<int64_t> e2i(ne);
    for (size_t e = 0; e < ne; ++e) e2i[(size_t)t.elem_int2ext[e]] = (int64_t)e;
    const size_t chunk = 1 << 14;
    const int64_t nc = (int64_t)((ne + chunk - 1) / chunk);
    std::vector<std::string> bufs((size_t)nc);
#pragma omp parallel for schedule(dynamic)
    for (int64_t c = 0; c < nc; ++c) {
      std::string& s = bufs[(size_t)c];
      char tmp[32];
      for (size_t E = (size_t)c * chunk; E < std::min(ne, (size_t)(c + 1) * chunk); ++E) {
        const int64_t e = e2i[E];
        for (int l = 0; l < 8; ++l) {
          const int k = std::snprintf(tmp, sizeof(tmp), "%10lu\t",
                                      (unsigned long)(t.node_int2ext[(size_t)nie[(size_t)e * 8 + l]] + 1));
          s.append(tmp, (size_t)k);
        }
        s.push_back('\n');
      }
    }
    for (auto& s : bufs) o->conn_text += s;
    char one[32], minus[32];
    std::snprintf(one, sizeof(one), "%12.5e\n", 1.0);
    std::snprintf(minus, sizeof(minus), "%12.5e\n", -1.0);
    o->switch_text.reserve(ne * 13);
    for (size_t E = 0; E < ne; ++E) o->switch_text += (E & 1) ? minus : one;
  }
  {
    long long cyc = 0;
    if (h->has_state) TRY(cycles_done(h, &cyc));
    o->t0_pending = h->has_state ? (cyc == 0) : true;
  }
  o->writer = std::thread(writer_loop, o);
  return fierro::rebuild_graphs(h);
}
