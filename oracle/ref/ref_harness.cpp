// Driver for the reference oracle build: the call sequence of
// Explicit-Lagrange-Kokkos/SGH_solver/driver.cpp:70-328 (input, mesh read,
// connectivity, dual views, get_vol, setup, sgh_solve) followed by a binary dump
// of the final state.  It also supplies write_outputs (outputs.cpp:10-78) as a
// no-op, since graphics dumps are outside the measured path, except in the
// fierro_ref_out build (-DFIERRO_REF_REAL_OUTPUTS), which links the reference's
// own outputs.cpp and writes its EnSight and state files into the working
// directory, and except in the fierro_ref_lib build (-DFIERRO_REF_CALL_LIBRARY),
// where the sgh_solve call is replaced by the reference-side binding of the GB300
// library (oracle/ref/fierro_sgh_call.inc: the same arrays to fierro_sgh_solve),
// linked against libfierro_sgh.so.  Linked only into the reference oracle
// executables built by oracle/build_ref.py.
//
// usage: fierro_ref <config.txt> <mesh.geo|mesh.bin> <state_out.bin>
// env FIERRO_REF_WARMUP=W runs W untimed cycles first (see main).
// The dump (little endian): "FSGHSTAT", u64 num_nodes, u64 num_elems,
// f64 time_value, then f64 arrays node_coords[2][Nn][D], node_vel[2][Nn][D],
// node_mass[Nn], elem_den[Ne], elem_pres[Ne], elem_sspd[Ne], elem_sie[2][Ne],
// elem_vol[Ne], elem_div[Ne], elem_mass[Ne], corner_force[2^D Ne][D] (D = num_dims),
// elem_stress[2][Ne][3][3], u64 num_state_vars, elem_statev[Ne][num_state_vars].
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "matar.h"
#include "mesh.h"
#include "state.h"
#ifdef FIERRO_REF_CALL_LIBRARY
#include <vector>

#include "fierro_sgh.h"
#endif

const char* fierro_ref_config_path = nullptr;

#ifndef FIERRO_REF_REAL_OUTPUTS
void write_outputs(const mesh_t& mesh, DViewCArrayKokkos<double>& node_coords,
                   DViewCArrayKokkos<double>& node_vel, DViewCArrayKokkos<double>& node_mass,
                   DViewCArrayKokkos<double>& elem_den, DViewCArrayKokkos<double>& elem_pres,
                   DViewCArrayKokkos<double>& elem_stress, DViewCArrayKokkos<double>& elem_sspd,
                   DViewCArrayKokkos<double>& elem_sie, DViewCArrayKokkos<double>& elem_vol,
                   DViewCArrayKokkos<double>& elem_mass, DViewCArrayKokkos<size_t>& elem_mat_id,
                   CArray<double>& graphics_times, size_t& graphics_id, const double time_value) {
  graphics_times(graphics_id) = time_value;
  graphics_id = (graphics_id + 1) % graphics_times.size();
}
#endif

static void put(FILE* f, const double* p, size_t n) { std::fwrite(p, sizeof(double), n, f); }

int main(int argc, char* argv[]) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: %s config.txt mesh state_out.bin\n", argv[0]);
    return 2;
  }
  fierro_ref_config_path = argv[1];
  size_t num_dims = 3, num_materials = 0, num_state_vars = 0, num_fills = 0, num_bcs = 0;
  size_t graphics_id = 0, graphics_cyc_ival = 50;
  CArray<double> graphics_times(2000);
  double graphics_dt_ival = 1.0e8, graphics_time = graphics_dt_ival;
  double time_value = 0.0, time_final = 1.e16, dt = 1.e-8, dt_max = 1.0e-2, dt_min = 1.0e-8;
  double dt_cfl = 0.4, dt_start = 1.0e-8;
  size_t rk_num_stages = 2, rk_num_bins = 2, cycle_stop = 1000000000;
  const double fuzz = 1.0e-16, tiny = 1.0e-12, small = 1.0e-8;  // driver.cpp:60-62

  Kokkos::initialize();
  {
    node_t node;
    elem_t elem;
    corner_t corner;
    CArrayKokkos<material_t> material;
    CArrayKokkos<double> state_vars;
    mesh_t mesh;
    CArrayKokkos<mat_fill_t> mat_fill;
    CArrayKokkos<boundary_t> boundary;

    input(material, mat_fill, boundary, state_vars, num_materials, num_fills, num_bcs, num_dims,
          num_state_vars, dt_start, time_final, dt_max, dt_min, dt_cfl, graphics_dt_ival,
          graphics_cyc_ival, cycle_stop, rk_num_stages);

    auto s0 = std::chrono::high_resolution_clock::now();
    read_mesh_ensight(argv[2], mesh, node, elem, corner, num_dims, rk_num_bins);
    mesh.build_corner_connectivity();
    mesh.build_elem_elem_connectivity();
    mesh.build_patch_connectivity();
    mesh.build_node_node_connectivity();

    const size_t num_nodes = mesh.num_nodes, num_elems = mesh.num_elems, num_corners = mesh.num_corners;
    elem.statev = CArray<double>(num_elems, num_state_vars);
    DViewCArrayKokkos<double> node_coords(&node.coords(0, 0, 0), rk_num_bins, num_nodes, num_dims);
    DViewCArrayKokkos<double> node_vel(&node.vel(0, 0, 0), rk_num_bins, num_nodes, num_dims);
    DViewCArrayKokkos<double> node_mass(&node.mass(0), num_nodes);
    DViewCArrayKokkos<double> elem_den(&elem.den(0), num_elems);
    DViewCArrayKokkos<double> elem_pres(&elem.pres(0), num_elems);
    DViewCArrayKokkos<double> elem_stress(&elem.stress(0, 0, 0, 0), rk_num_bins, num_elems, 3, 3);
    DViewCArrayKokkos<double> elem_sspd(&elem.sspd(0), num_elems);
    DViewCArrayKokkos<double> elem_sie(&elem.sie(0, 0), rk_num_bins, num_elems);
    DViewCArrayKokkos<double> elem_vol(&elem.vol(0), num_elems);
    DViewCArrayKokkos<double> elem_div(&elem.div(0), num_elems);
    DViewCArrayKokkos<double> elem_mass(&elem.mass(0), num_elems);
    DViewCArrayKokkos<size_t> elem_mat_id(&elem.mat_id(0), num_elems);
    DViewCArrayKokkos<double> elem_statev(&elem.statev(0, 0), num_elems, num_state_vars);
    DViewCArrayKokkos<double> corner_force(&corner.force(0, 0), num_corners, num_dims);
    DViewCArrayKokkos<double> corner_mass(&corner.mass(0), num_corners);

    get_vol(elem_vol, node_coords, mesh);
    setup(material, mat_fill, boundary, mesh, node_coords, node_vel, node_mass, elem_den, elem_pres,
          elem_stress, elem_sspd, elem_sie, elem_vol, elem_mass, elem_mat_id, elem_statev, state_vars,
          corner_mass, num_fills, rk_num_bins, num_bcs, num_materials, num_state_vars);
    auto s1 = std::chrono::high_resolution_clock::now();
    std::printf("Setup time in seconds: %f\n",
                std::chrono::duration_cast<std::chrono::nanoseconds>(s1 - s0).count() * 1e-9);

    time_value = 0.0;
    dt = dt_start;
    graphics_id = 0;
    graphics_times(0) = 0.0;
    graphics_time = graphics_dt_ival;

    // optional untimed warm-up cycles (FIERRO_REF_WARMUP=W): a first sgh_solve call of
    // W cycles, after which the deck's cycle_stop cycles run as a second call whose
    // printed "Calculation time" is the timed one
    const char* warm = std::getenv("FIERRO_REF_WARMUP");
    const size_t warm_cycles = warm ? (size_t)std::strtoull(warm, nullptr, 10) : 0;
    if (warm_cycles > 0)
      sgh_solve(material, boundary, mesh, node_coords, node_vel, node_mass, elem_den, elem_pres,
                elem_stress, elem_sspd, elem_sie, elem_vol, elem_div, elem_mass, elem_mat_id,
                elem_statev, corner_force, corner_mass, time_value, time_final, dt_max, dt_min, dt_cfl,
                graphics_time, graphics_cyc_ival, graphics_dt_ival, warm_cycles, rk_num_stages, dt, fuzz,
                tiny, small, graphics_times, graphics_id);

#ifdef FIERRO_REF_CALL_LIBRARY
    // the reference-side binding of the GB300 library, verbatim (the snippet the
    // integration notes show): the same host arrays go to fierro_sgh_solve
    {
#include "fierro_sgh_call.inc"
    }
#else
    sgh_solve(material, boundary, mesh, node_coords, node_vel, node_mass, elem_den, elem_pres,
              elem_stress, elem_sspd, elem_sie, elem_vol, elem_div, elem_mass, elem_mat_id,
              elem_statev, corner_force, corner_mass, time_value, time_final, dt_max, dt_min, dt_cfl,
              graphics_time, graphics_cyc_ival, graphics_dt_ival, cycle_stop, rk_num_stages, dt, fuzz,
              tiny, small, graphics_times, graphics_id);
#endif

    FILE* f = std::fopen(argv[3], "wb");
    if (!f) return 3;
    const uint64_t hdr[2] = {num_nodes, num_elems};
    std::fwrite("FSGHSTAT", 1, 8, f);
    std::fwrite(hdr, sizeof(uint64_t), 2, f);
    put(f, &time_value, 1);
    put(f, &node.coords(0, 0, 0), rk_num_bins * num_nodes * num_dims);
    put(f, &node.vel(0, 0, 0), rk_num_bins * num_nodes * num_dims);
    put(f, &node.mass(0), num_nodes);
    put(f, &elem.den(0), num_elems);
    put(f, &elem.pres(0), num_elems);
    put(f, &elem.sspd(0), num_elems);
    put(f, &elem.sie(0, 0), rk_num_bins * num_elems);
    put(f, &elem.vol(0), num_elems);
    put(f, &elem.div(0), num_elems);
    put(f, &elem.mass(0), num_elems);
    put(f, &corner.force(0, 0), num_corners * num_dims);
    put(f, &elem.stress(0, 0, 0, 0), rk_num_bins * num_elems * 9);
    const uint64_t nsv = num_state_vars;
    std::fwrite(&nsv, sizeof(uint64_t), 1, f);
    put(f, &elem.statev(0, 0), num_elems * num_state_vars);
    std::fclose(f);
  }
  Kokkos::finalize();
  return 0;
}
