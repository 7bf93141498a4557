// Golden-vector driver for the omega_playground reference sources.
//
// Test infrastructure only: it links the reference's own, unmodified
// src/mesh, src/model and src/time_integration sources (compiled against the
// host-only Kokkos shim in oracle/kokkos_shim) and runs one scenario read from
// a file of named arrays.  It writes the mesh tables, every auxiliary field and
// tendency after one ShallowWaterModel::compute_tendency on the initial state,
// the three diagnostics, and the state after `nsteps` steps of the requested
// time stepper.  Reference call sites followed:
//   mesh        src/mesh/planar_hexagonal_mesh.cpp:8-62
//   model       src/model/shallow_water_model.cpp:5-41, 313-347
//   steppers    src/time_integration/rk4.cpp:28-104, lsrk.cpp:36-89
//   diagnostics src/model/shallow_water_diagnostics.cpp:5-89
//
// File format (both directions): repeated records of
//   char name[32]; char dtype ('d' or 'i'); int32 ndim; int64 dims[ndim]; data
#include <omega.hpp>

#include <cstdio>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

using namespace omega;

namespace {

struct Array {
  char dtype = 'd';
  std::vector<long> dims;
  std::vector<double> d;
  std::vector<int> i;
};

std::map<std::string, Array> read_file(const char *path) {
  std::map<std::string, Array> out;
  FILE *f = std::fopen(path, "rb");
  if (!f)
    throw std::runtime_error(std::string("cannot open ") + path);
  char name[32];
  while (std::fread(name, 1, 32, f) == 32) {
    Array a;
    int ndim = 0;
    if (std::fread(&a.dtype, 1, 1, f) != 1 || std::fread(&ndim, 4, 1, f) != 1)
      throw std::runtime_error("truncated header");
    a.dims.resize(ndim);
    long n = 1;
    for (int r = 0; r < ndim; ++r) {
      long long dd;
      if (std::fread(&dd, 8, 1, f) != 1)
        throw std::runtime_error("truncated dims");
      a.dims[r] = long(dd);
      n *= a.dims[r];
    }
    if (a.dtype == 'd') {
      a.d.resize(n);
      if (n && std::fread(a.d.data(), 8, n, f) != size_t(n))
        throw std::runtime_error("truncated data");
    } else {
      a.i.resize(n);
      if (n && std::fread(a.i.data(), 4, n, f) != size_t(n))
        throw std::runtime_error("truncated data");
    }
    name[31] = 0;
    out[name] = a;
  }
  std::fclose(f);
  return out;
}

struct Writer {
  FILE *f;
  explicit Writer(const char *path) : f(std::fopen(path, "wb")) {
    if (!f)
      throw std::runtime_error(std::string("cannot open ") + path);
  }
  ~Writer() { std::fclose(f); }
  void header(const char *name, char dtype, const std::vector<long> &dims) {
    char buf[32] = {0};
    std::strncpy(buf, name, 31);
    std::fwrite(buf, 1, 32, f);
    std::fwrite(&dtype, 1, 1, f);
    int nd = int(dims.size());
    std::fwrite(&nd, 4, 1, f);
    for (long d : dims) {
      long long dd = d;
      std::fwrite(&dd, 8, 1, f);
    }
  }
  template <class V> void view(const char *name, const V &v) {
    std::vector<long> dims;
    for (int r = 0; r < V::rank; ++r)
      dims.push_back(long(v.extent(r)));
    using T = typename V::non_const_value_type;
    header(name, std::is_same<T, double>::value ? 'd' : 'i', dims);
    std::fwrite(v.data(), sizeof(T), v.size(), f);
  }
  void scalar(const char *name, double x) {
    header(name, 'd', {1});
    std::fwrite(&x, 8, 1, f);
  }
};

template <class V> void fill(const V &v, const Array &a) {
  if (a.d.size() != v.size())
    throw std::runtime_error("size mismatch for " + v.label());
  for (size_t n = 0; n < v.size(); ++n)
    v.data()[n] = a.d[n];
}

} // namespace

int main(int argc, char **argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s input.bin output.bin\n", argv[0]);
    return 2;
  }
  Kokkos::initialize();
  auto in = read_file(argv[1]);
  const auto &pi = in.at("params_i").i;
  const auto &pd = in.at("params_d").d;
  const Int nx = pi[0], ny = pi[1], nlayers = pi[2], ntracers = pi[3];
  const Int stepper_kind = pi[4], nsteps = pi[5];

  PlanarHexagonalMesh mesh(nx, ny, pd[0], nlayers);
  ShallowWaterParams params;
  params.m_f0 = pd[1];
  params.m_grav = pd[2];
  params.m_visc_del2 = pd[3];
  params.m_visc_del4 = pd[4];
  params.m_eddy_diff2 = pd[5];
  params.m_eddy_diff4 = pd[6];
  params.m_ntracers = ntracers;
  params.m_disable_h_tendency = pi[6] != 0;
  params.m_disable_vn_tendency = pi[7] != 0;
  const Real dt = pd[7], t0 = pd[8];

  ShallowWaterModel model(&mesh, params);
  ShallowWaterState state(&mesh, params);
  fill(state.m_h_cell, in.at("h"));
  fill(state.m_vn_edge, in.at("vn"));
  if (ntracers > 0)
    fill(state.m_tr_cell, in.at("tr"));

  Writer w(argv[2]);
  // mesh tables
  w.view("nedges_on_cell", mesh.m_nedges_on_cell);
  w.view("edges_on_cell", mesh.m_edges_on_cell);
  w.view("cells_on_cell", mesh.m_cells_on_cell);
  w.view("vertices_on_cell", mesh.m_vertices_on_cell);
  w.view("kite_index_on_cell", mesh.m_kite_index_on_cell);
  w.view("nedges_on_edge", mesh.m_nedges_on_edge);
  w.view("edges_on_edge", mesh.m_edges_on_edge);
  w.view("cells_on_edge", mesh.m_cells_on_edge);
  w.view("vertices_on_edge", mesh.m_vertices_on_edge);
  w.view("edges_on_vertex", mesh.m_edges_on_vertex);
  w.view("cells_on_vertex", mesh.m_cells_on_vertex);
  w.view("area_cell", mesh.m_area_cell);
  w.view("x_cell", mesh.m_x_cell);
  w.view("y_cell", mesh.m_y_cell);
  w.view("edge_sign_on_cell", mesh.m_edge_sign_on_cell);
  w.view("dc_edge", mesh.m_dc_edge);
  w.view("dv_edge", mesh.m_dv_edge);
  w.view("angle_edge", mesh.m_angle_edge);
  w.view("x_edge", mesh.m_x_edge);
  w.view("y_edge", mesh.m_y_edge);
  w.view("weights_on_edge", mesh.m_weights_on_edge);
  w.view("area_triangle", mesh.m_area_triangle);
  w.view("x_vertex", mesh.m_x_vertex);
  w.view("y_vertex", mesh.m_y_vertex);
  w.view("kiteareas_on_vertex", mesh.m_kiteareas_on_vertex);
  w.view("edge_sign_on_vertex", mesh.m_edge_sign_on_vertex);

  // diagnostics on the initial state
  w.scalar("mass0", mass_integral(state, model));
  w.scalar("energy0", energy_integral(state, model));
  w.scalar("circulation0", circulation_integral(state, model));

  // one tendency evaluation (replace) and every auxiliary field it produced
  ShallowWaterState tend(&mesh, params);
  model.compute_tendency(tend, state, t0);
  const auto &aux = model.m_aux_state;
  w.view("rvort_vertex", aux.m_vorticity_aux.m_rvort_vertex);
  w.view("norm_rvort_vertex", aux.m_vorticity_aux.m_norm_rvort_vertex);
  w.view("norm_pvort_vertex", aux.m_vorticity_aux.m_norm_pvort_vertex);
  w.view("norm_rvort_edge", aux.m_vorticity_aux.m_norm_rvort_edge);
  w.view("norm_pvort_edge", aux.m_vorticity_aux.m_norm_pvort_edge);
  w.view("mean_h_edge", aux.m_thickness_aux.m_mean_h_edge);
  w.view("ke_cell", aux.m_kinetic_aux.m_ke_cell);
  w.view("vel_div_cell", aux.m_kinetic_aux.m_vel_div_cell);
  w.view("norm_tr_cell", aux.m_tracer_aux.m_norm_tr_cell);
  w.view("vel_del2_edge", model.m_vel_hyperdiff_edge.m_vel_del2_edge);
  w.view("vel_del2_rvort_vertex",
         model.m_vel_hyperdiff_edge.m_vel_del2_rvort_vertex);
  w.view("vel_del2_div_cell", model.m_vel_hyperdiff_edge.m_vel_del2_div_cell);
  w.view("tracer_del2_cell", model.m_tracer_hyperdiff_cell.m_tracer_del2_cell);
  w.view("tend_h", tend.m_h_cell);
  w.view("tend_vn", tend.m_vn_edge);
  w.view("tend_tr", tend.m_tr_cell);

  // time stepping
  if (stepper_kind != 0 && nsteps > 0) {
    std::unique_ptr<TimeStepper> stepper;
    if (stepper_kind == 1)
      stepper = std::make_unique<RK4Stepper>(model);
    else if (stepper_kind == 2)
      stepper = std::make_unique<LSRKStepper>(model, 5);
    else
      stepper = std::make_unique<LSRKStepper>(model, 1);
    for (Int s = 0; s < nsteps; ++s)
      stepper->do_step(t0 + s * dt, dt, state);
  }
  w.view("h_final", state.m_h_cell);
  w.view("vn_final", state.m_vn_edge);
  w.view("tr_final", state.m_tr_cell);
  w.scalar("mass1", mass_integral(state, model));
  w.scalar("energy1", energy_integral(state, model));
  w.scalar("circulation1", circulation_integral(state, model));
  Kokkos::finalize();
  return 0;
}
