// Config-driven replacement for Explicit-Lagrange-Kokkos/SGH_solver/input.cpp,
// the same input-swap mechanism the reference's own
// tests-for-Explicit-Lagrange-Kokkos/input_for_*.cpp files use.  Linked only into
// the reference oracle build (oracle/build_ref.py), never into the library.
//
// The problem is read from the text file named by fierro_ref_config_path:
//   <key> <value>                    scalar controls (dt_start, time_final, ...,
//                                    num_dims 2 for the 2D-RZ path)
//   material q1 q1ex q2 q2ex sv0 .. sv{num_state_vars-1}
//   fill volume mat_id x1 x2 y1 y2 z1 z2 r1 r2 velocity u v w speed sie den
//   bc surface value hydro_bc
//   strength mat_id type             type 1 = hypo, 2 = hyper: the material runs
//                                    fierro_test_strength_model (ref_user_mat.cpp)
// Numbers are parsed with strtod, so a %.17g (or hex-float) value round-trips.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "matar.h"
#include "mesh.h"
#include "state.h"

extern const char* fierro_ref_config_path;

void fierro_test_strength_model(const DViewCArrayKokkos<double>& elem_pres,
                                const DViewCArrayKokkos<double>& elem_stress, const size_t elem_gid,
                                const size_t mat_id, const DViewCArrayKokkos<double>& elem_state_vars,
                                const DViewCArrayKokkos<double>& elem_sspd, const double den, const double sie,
                                const ViewCArrayKokkos<double>& vel_grad,
                                const ViewCArrayKokkos<size_t>& elem_node_gids,
                                const DViewCArrayKokkos<double>& node_coords,
                                const DViewCArrayKokkos<double>& node_vel, const double vol, const double dt,
                                const double rk_alpha);

namespace {

struct MatRec { double q1, q1ex, q2, q2ex; std::vector<double> sv; };
struct FillRec { double v[17]; };
struct BcRec { int surface; double value; int hydro; };

std::vector<std::string> tokens(const std::string& line) {
  std::vector<std::string> out;
  size_t i = 0;
  while (i < line.size()) {
    while (i < line.size() && (line[i] == ' ' || line[i] == '\t' || line[i] == '\r')) ++i;
    size_t j = i;
    while (j < line.size() && line[j] != ' ' && line[j] != '\t' && line[j] != '\r') ++j;
    if (j > i) out.push_back(line.substr(i, j - i));
    i = j;
  }
  return out;
}

double num(const std::string& s) { return std::strtod(s.c_str(), nullptr); }

}  // namespace

void input(CArrayKokkos<material_t>& material, CArrayKokkos<mat_fill_t>& mat_fill,
           CArrayKokkos<boundary_t>& boundary, CArrayKokkos<double>& state_vars,
           size_t& num_materials, size_t& num_fills, size_t& num_bcs, size_t& num_dims,
           size_t& max_num_state_vars, double& dt_start, double& time_final, double& dt_max,
           double& dt_min, double& dt_cfl, double& graphics_dt_ival, size_t& graphics_cyc_ival,
           size_t& cycle_stop, size_t& rk_num_stages) {
  FILE* f = std::fopen(fierro_ref_config_path, "r");
  if (!f) {
    std::fprintf(stderr, "cannot open config %s\n", fierro_ref_config_path);
    std::exit(2);
  }
  num_dims = 3;
  max_num_state_vars = 6;
  std::vector<MatRec> mats;
  std::vector<FillRec> fills;
  std::vector<BcRec> bcs;
  std::vector<std::pair<size_t, int>> strengths;
  char buf[4096];
  while (std::fgets(buf, sizeof(buf), f)) {
    std::string line(buf);
    if (!line.empty() && line.back() == '\n') line.pop_back();
    auto t = tokens(line);
    if (t.empty() || t[0][0] == '#') continue;
    const std::string& k = t[0];
    if (k == "dt_start") dt_start = num(t[1]);
    else if (k == "time_final") time_final = num(t[1]);
    else if (k == "dt_max") dt_max = num(t[1]);
    else if (k == "dt_min") dt_min = num(t[1]);
    else if (k == "dt_cfl") dt_cfl = num(t[1]);
    else if (k == "graphics_dt_ival") graphics_dt_ival = num(t[1]);
    else if (k == "graphics_cyc_ival") graphics_cyc_ival = (size_t)std::strtoull(t[1].c_str(), nullptr, 10);
    else if (k == "cycle_stop") cycle_stop = (size_t)std::strtoull(t[1].c_str(), nullptr, 10);
    else if (k == "rk_num_stages") rk_num_stages = (size_t)std::strtoull(t[1].c_str(), nullptr, 10);
    else if (k == "num_state_vars") max_num_state_vars = (size_t)std::strtoull(t[1].c_str(), nullptr, 10);
    else if (k == "num_dims") num_dims = (size_t)std::strtoull(t[1].c_str(), nullptr, 10);
    else if (k == "material") {
      MatRec m{num(t[1]), num(t[2]), num(t[3]), num(t[4]), {}};
      for (size_t i = 5; i < t.size(); ++i) m.sv.push_back(num(t[i]));
      mats.push_back(m);
    } else if (k == "fill") {
      FillRec r{};
      for (size_t i = 1; i < t.size() && i <= 17; ++i) r.v[i - 1] = num(t[i]);
      fills.push_back(r);
    } else if (k == "bc") {
      bcs.push_back(BcRec{(int)num(t[1]), num(t[2]), (int)num(t[3])});
    } else if (k == "strength") {
      strengths.emplace_back((size_t)num(t[1]), (int)num(t[2]));
    }
  }
  std::fclose(f);

  num_materials = mats.size();
  material = CArrayKokkos<material_t>(num_materials);
  state_vars = CArrayKokkos<double>(num_materials, max_num_state_vars);
  num_fills = fills.size();
  mat_fill = CArrayKokkos<mat_fill_t>(num_fills);
  num_bcs = bcs.size();
  boundary = CArrayKokkos<boundary_t>(num_bcs);

  for (size_t m = 0; m < num_materials; ++m) {
    material(m).eos_model = ideal_gas;
    material(m).strength_type = model::none;
    material(m).strength_setup = model_init::input;
    material(m).strength_model = NULL;
    material(m).q1 = mats[m].q1;
    material(m).q1ex = mats[m].q1ex;
    material(m).q2 = mats[m].q2;
    material(m).q2ex = mats[m].q2ex;
    material(m).num_state_vars = max_num_state_vars;
    for (size_t v = 0; v < max_num_state_vars && v < mats[m].sv.size(); ++v) state_vars(m, v) = mats[m].sv[v];
  }
  for (const auto& st : strengths) {
    if (st.first >= num_materials || st.second < 1 || st.second > 2) {
      std::fprintf(stderr, "bad strength line: material %zu type %d\n", st.first, st.second);
      std::exit(2);
    }
    material(st.first).strength_type = (model::strength_tag)st.second;
    material(st.first).strength_model = fierro_test_strength_model;
  }
  for (size_t i = 0; i < num_fills; ++i) {
    const double* v = fills[i].v;
    mat_fill(i).volume = (region::vol_tag)(int)v[0];
    mat_fill(i).mat_id = (size_t)v[1];
    mat_fill(i).x1 = v[2];
    mat_fill(i).x2 = v[3];
    mat_fill(i).y1 = v[4];
    mat_fill(i).y2 = v[5];
    mat_fill(i).z1 = v[6];
    mat_fill(i).z2 = v[7];
    mat_fill(i).radius1 = v[8];
    mat_fill(i).radius2 = v[9];
    mat_fill(i).velocity = (init_conds::init_velocity_conds)(int)v[10];
    mat_fill(i).u = v[11];
    mat_fill(i).v = v[12];
    mat_fill(i).w = v[13];
    mat_fill(i).speed = v[14];
    mat_fill(i).sie = v[15];
    mat_fill(i).den = v[16];
  }
  for (size_t i = 0; i < num_bcs; ++i) {
    boundary(i).surface = (bdy::bdy_tag)bcs[i].surface;
    boundary(i).value = bcs[i].value;
    boundary(i).hydro_bc = (bdy::bdy_hydro_conds)bcs[i].hydro;
  }
}
