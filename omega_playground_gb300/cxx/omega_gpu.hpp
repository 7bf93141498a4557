// omega_gpu.hpp - C++ drop-in for omega_playground's mesh, state, model and
// time-stepper classes, running on the GB300 CUDA library (libswgpu.so)
// through the C ABI in swgpu.h.
//
// Names and signatures follow the reference (paths inside its checkout):
//   MPASMesh, PlanarHexagonalMesh      src/mesh/mpas_mesh.hpp:7-71,
//                                      src/mesh/planar_hexagonal_mesh.hpp:8-28
//   ShallowWaterParams                 src/model/shallow_water_params.hpp:7-18
//   ShallowWaterState                  src/model/shallow_water_state.hpp:9-16
//   ShallowWaterModel, AddMode         src/model/shallow_water_model.hpp:11-51
//   TimeStepper, LSRKStepper, RK4Stepper
//                                      src/time_integration/time_stepper.hpp:8-38
//   energy/mass/circulation_integral   src/model/shallow_water_diagnostics.hpp:7-12
//   LinearShallowWaterModel/Params     src/shallow_water_hierarchical.cpp:676-775
//                                      (never built in the reference)
//
// Differences a reference user sees:
//  - Real1d/Real2d/Real3d are DeviceView (a device pointer plus extents,
//    LayoutRight), usable inside the user's own __global__ kernels, instead
//    of Kokkos::View.  Mesh tables are host std::vector members with the
//    reference's names (m_x_cell, m_angle_edge, ...); device copies of the
//    geometry a forcing kernel needs are available as d_* members.
//  - ShallowWaterModel::additional_tendency receives DeviceViews and runs on
//    the library's stream (the legacy default stream here); an override
//    launches its own kernel.
//  - Errors throw std::runtime_error with the library's message.
#pragma once

#include <swgpu.h>

#include <cuda_runtime.h>

#include <cmath>
#include <exception>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <typeinfo>
#include <vector>

namespace omega {

using Real = double;
using Int = int;
constexpr Real pi = 3.14159265358979323846;
constexpr Int vector_length = 1;

inline void swg_check(int rc) {
  if (rc != SWG_OK)
    throw std::runtime_error(std::string("swgpu: ") + swg_last_error());
}

inline void fence() { swg_check(swg_sync(nullptr)); }

// Non-owning view of device memory, LayoutRight like the reference's Views.
template <class T, int R> struct DeviceView {
  T *m_data = nullptr;
  Int m_ext[R] = {};
  __host__ __device__ T &operator()(Int i) const { return m_data[i]; }
  __host__ __device__ T &operator()(Int i, Int j) const {
    return m_data[size_t(i) * m_ext[1] + j];
  }
  __host__ __device__ T &operator()(Int i, Int j, Int k) const {
    return m_data[(size_t(i) * m_ext[1] + j) * m_ext[2] + k];
  }
  __host__ __device__ Int extent(int r) const { return m_ext[r]; }
  __host__ __device__ T *data() const { return m_data; }
  size_t size() const {
    size_t n = 1;
    for (int r = 0; r < R; ++r)
      n *= size_t(m_ext[r]);
    return n;
  }
  // a view of mutable elements converts to a read-only view
  template <class U = T,
            class = typename std::enable_if<!std::is_const<U>::value>::type>
  operator DeviceView<const U, R>() const {
    DeviceView<const U, R> v;
    v.m_data = m_data;
    for (int r = 0; r < R; ++r)
      v.m_ext[r] = m_ext[r];
    return v;
  }
};
using Real1d = DeviceView<Real, 1>;
using Real2d = DeviceView<Real, 2>;
using Real3d = DeviceView<Real, 3>;
using RealConst1d = DeviceView<const Real, 1>;
using RealConst2d = DeviceView<const Real, 2>;
using RealConst3d = DeviceView<const Real, 3>;

// Owning device array (cudaMalloc / cudaFree) with host round trips.
template <class T> class DeviceArray {
public:
  DeviceArray() = default;
  explicit DeviceArray(const std::vector<T> &host) { assign(host); }
  DeviceArray(const DeviceArray &) = delete;
  DeviceArray &operator=(const DeviceArray &) = delete;
  ~DeviceArray() { cudaFree(m_ptr); }
  void assign(const std::vector<T> &host) {
    cudaFree(m_ptr);
    m_ptr = nullptr;
    m_n = host.size();
    if (cudaMalloc(&m_ptr, std::max<size_t>(m_n, 1) * sizeof(T)) != cudaSuccess)
      throw std::runtime_error("DeviceArray: cudaMalloc failed");
    if (m_n && cudaMemcpy(m_ptr, host.data(), m_n * sizeof(T),
                          cudaMemcpyHostToDevice) != cudaSuccess)
      throw std::runtime_error("DeviceArray: cudaMemcpy failed");
  }
  T *data() const { return m_ptr; }
  size_t size() const { return m_n; }
  DeviceView<T, 1> view() const {
    DeviceView<T, 1> v;
    v.m_data = m_ptr;
    v.m_ext[0] = Int(m_n);
    return v;
  }

private:
  T *m_ptr = nullptr;
  size_t m_n = 0;
};

// ------------------------------------------------------------------- mesh --

struct MPASMesh {
  static constexpr Int maxedges = 6;
  Int m_nlayers = 0, m_nlayers_vec = 0, m_ncells = 0, m_nedges = 0,
      m_nvertices = 0;

  std::vector<Int> m_nedges_on_cell, m_edges_on_cell, m_cells_on_cell,
      m_vertices_on_cell, m_kite_index_on_cell;
  std::vector<Real> m_area_cell, m_x_cell, m_y_cell, m_edge_sign_on_cell;
  std::vector<Int> m_nedges_on_edge, m_edges_on_edge, m_cells_on_edge,
      m_vertices_on_edge;
  std::vector<Real> m_dc_edge, m_dv_edge, m_angle_edge, m_x_edge, m_y_edge,
      m_weights_on_edge, m_mesh_scaling_del2, m_mesh_scaling_del4,
      m_edge_mask;
  std::vector<Int> m_edges_on_vertex, m_cells_on_vertex;
  std::vector<Real> m_area_triangle, m_x_vertex, m_y_vertex,
      m_kiteareas_on_vertex, m_edge_sign_on_vertex;
  // levels per column for the diagnostics; empty = m_nlayers everywhere
  std::vector<Int> m_max_level_cell, m_max_level_vertex_bot;

  // device copies of the geometry user kernels typically read
  DeviceArray<Real> d_x_cell, d_y_cell, d_x_edge, d_y_edge, d_angle_edge;

  swg_mesh m_handle = nullptr;

  MPASMesh() = default;
  MPASMesh(const MPASMesh &) = delete;
  MPASMesh &operator=(const MPASMesh &) = delete;
  virtual ~MPASMesh() { swg_mesh_destroy(m_handle); }

  // Uploads the tables (MPASMesh::finalize_mesh, mpas_mesh.cpp:5-57: scaling
  // and mask default to ones when left empty).
  void finalize_mesh() {
    swg_mesh_desc d{};
    d.ncells = m_ncells;
    d.nedges = m_nedges;
    d.nvertices = m_nvertices;
    d.nlayers = m_nlayers;
    d.nedges_on_cell = m_nedges_on_cell.data();
    d.edges_on_cell = m_edges_on_cell.data();
    d.nedges_on_edge = m_nedges_on_edge.data();
    d.edges_on_edge = m_edges_on_edge.data();
    d.cells_on_edge = m_cells_on_edge.data();
    d.vertices_on_edge = m_vertices_on_edge.data();
    d.edges_on_vertex = m_edges_on_vertex.data();
    d.cells_on_vertex = m_cells_on_vertex.data();
    d.area_cell = m_area_cell.data();
    d.edge_sign_on_cell = m_edge_sign_on_cell.data();
    d.dc_edge = m_dc_edge.data();
    d.dv_edge = m_dv_edge.data();
    d.weights_on_edge = m_weights_on_edge.data();
    d.area_triangle = m_area_triangle.data();
    d.kiteareas_on_vertex = m_kiteareas_on_vertex.data();
    d.edge_sign_on_vertex = m_edge_sign_on_vertex.data();
    d.mesh_scaling_del2 =
        m_mesh_scaling_del2.empty() ? nullptr : m_mesh_scaling_del2.data();
    d.mesh_scaling_del4 =
        m_mesh_scaling_del4.empty() ? nullptr : m_mesh_scaling_del4.data();
    d.edge_mask = m_edge_mask.empty() ? nullptr : m_edge_mask.data();
    d.max_level_cell =
        m_max_level_cell.empty() ? nullptr : m_max_level_cell.data();
    d.max_level_vertex_bot =
        m_max_level_vertex_bot.empty() ? nullptr : m_max_level_vertex_bot.data();
    swg_mesh_destroy(m_handle);
    m_handle = nullptr;
    swg_check(swg_mesh_create(&d, &m_handle));
    if (!m_x_cell.empty())
      d_x_cell.assign(m_x_cell);
    if (!m_y_cell.empty())
      d_y_cell.assign(m_y_cell);
    if (!m_x_edge.empty())
      d_x_edge.assign(m_x_edge);
    if (!m_y_edge.empty())
      d_y_edge.assign(m_y_edge);
    if (!m_angle_edge.empty())
      d_angle_edge.assign(m_angle_edge);
  }
};

struct PlanarHexagonalMesh : MPASMesh {
  Int m_nx, m_ny;
  Real m_dc, m_period_x, m_period_y;

  // True for odd ny: the half-cell shift of alternate rows does not
  // alternate across the periodic y boundary, so the reference's parallel
  // construction writes some table slots twice (a race) and the rows meet
  // irregularly there.  The tables are the reference's serial result.
  bool odd_row_seam() const { return m_ny % 2 == 1; }

  PlanarHexagonalMesh(Int nx, Int ny, Int nlayers = 1)
      : PlanarHexagonalMesh(nx, ny, 1. / nx, nlayers) {}
  PlanarHexagonalMesh(Int nx, Int ny, Real dc, Int nlayers = 1)
      : m_nx(nx), m_ny(ny), m_dc(dc) {
    m_nlayers = nlayers;
    m_nlayers_vec = nlayers;
    m_ncells = nx * ny;
    m_nedges = 3 * m_ncells;
    m_nvertices = 2 * m_ncells;
    const size_t C = m_ncells, E = m_nedges, V = m_nvertices;
    m_nedges_on_cell.resize(C);
    m_edges_on_cell.resize(6 * C);
    m_cells_on_cell.resize(6 * C);
    m_vertices_on_cell.resize(6 * C);
    m_kite_index_on_cell.resize(6 * C);
    m_area_cell.resize(C);
    m_x_cell.resize(C);
    m_y_cell.resize(C);
    m_edge_sign_on_cell.resize(6 * C);
    m_nedges_on_edge.resize(E);
    m_edges_on_edge.resize(12 * E);
    m_cells_on_edge.resize(2 * E);
    m_vertices_on_edge.resize(2 * E);
    m_dc_edge.resize(E);
    m_dv_edge.resize(E);
    m_angle_edge.resize(E);
    m_x_edge.resize(E);
    m_y_edge.resize(E);
    m_weights_on_edge.resize(12 * E);
    m_edges_on_vertex.resize(3 * V);
    m_cells_on_vertex.resize(3 * V);
    m_area_triangle.resize(V);
    m_x_vertex.resize(V);
    m_y_vertex.resize(V);
    m_kiteareas_on_vertex.resize(3 * V);
    m_edge_sign_on_vertex.resize(3 * V);
    swg_hex_tables t{};
    t.nedges_on_cell = m_nedges_on_cell.data();
    t.edges_on_cell = m_edges_on_cell.data();
    t.cells_on_cell = m_cells_on_cell.data();
    t.vertices_on_cell = m_vertices_on_cell.data();
    t.kite_index_on_cell = m_kite_index_on_cell.data();
    t.nedges_on_edge = m_nedges_on_edge.data();
    t.edges_on_edge = m_edges_on_edge.data();
    t.cells_on_edge = m_cells_on_edge.data();
    t.vertices_on_edge = m_vertices_on_edge.data();
    t.edges_on_vertex = m_edges_on_vertex.data();
    t.cells_on_vertex = m_cells_on_vertex.data();
    t.area_cell = m_area_cell.data();
    t.x_cell = m_x_cell.data();
    t.y_cell = m_y_cell.data();
    t.edge_sign_on_cell = m_edge_sign_on_cell.data();
    t.dc_edge = m_dc_edge.data();
    t.dv_edge = m_dv_edge.data();
    t.angle_edge = m_angle_edge.data();
    t.x_edge = m_x_edge.data();
    t.y_edge = m_y_edge.data();
    t.weights_on_edge = m_weights_on_edge.data();
    t.area_triangle = m_area_triangle.data();
    t.x_vertex = m_x_vertex.data();
    t.y_vertex = m_y_vertex.data();
    t.kiteareas_on_vertex = m_kiteareas_on_vertex.data();
    t.edge_sign_on_vertex = m_edge_sign_on_vertex.data();
    swg_check(swg_planar_hex_mesh_build(nx, ny, dc, &t, &m_period_x,
                                        &m_period_y));
    finalize_mesh();
  }
};

// ------------------------------------------------------------------ model --

struct ShallowWaterParams {
  Real m_f0;
  Real m_grav = 9.81;
  Real m_drag_coeff = 0;
  Real m_visc_del2 = 0;
  Real m_visc_del4 = 0;
  Real m_eddy_diff2 = 0;
  Real m_eddy_diff4 = 0;
  Int m_ntracers = 0;
  bool m_disable_h_tendency = false;
  bool m_disable_vn_tendency = false;
};

struct ShallowWaterState {
  std::shared_ptr<swg_state_s> m_handle;
  Real2d m_h_cell;
  Real2d m_vn_edge;
  Real3d m_tr_cell;

  ShallowWaterState(const MPASMesh *mesh, Int ntracers) {
    swg_state s = nullptr;
    swg_check(swg_state_create(mesh->m_handle, ntracers, &s));
    m_handle.reset(s, [](swg_state p) { swg_state_destroy(p); });
    double *h, *vn, *tr;
    swg_check(swg_state_device_ptrs(s, &h, &vn, &tr));
    m_h_cell.m_data = h;
    m_h_cell.m_ext[0] = mesh->m_ncells;
    m_h_cell.m_ext[1] = mesh->m_nlayers;
    m_vn_edge.m_data = vn;
    m_vn_edge.m_ext[0] = mesh->m_nedges;
    m_vn_edge.m_ext[1] = mesh->m_nlayers;
    m_tr_cell.m_data = tr;
    m_tr_cell.m_ext[0] = ntracers;
    m_tr_cell.m_ext[1] = mesh->m_ncells;
    m_tr_cell.m_ext[2] = mesh->m_nlayers;
  }
  ShallowWaterState(const MPASMesh *mesh, const ShallowWaterParams &params)
      : ShallowWaterState(mesh, params.m_ntracers) {}

  swg_state handle() const { return m_handle.get(); }
  // host round trips (reference users filled Views with parallel_for)
  void upload(const std::vector<Real> &h, const std::vector<Real> &vn,
              const std::vector<Real> &tr = {}) const {
    swg_check(swg_state_upload(handle(), h.data(), vn.data(),
                               tr.empty() ? nullptr : tr.data(), nullptr));
    fence();
  }
  void download(std::vector<Real> &h, std::vector<Real> &vn,
                std::vector<Real> &tr) const {
    h.resize(m_h_cell.size());
    vn.resize(m_vn_edge.size());
    tr.resize(m_tr_cell.size());
    swg_check(swg_state_download(handle(), h.data(), vn.data(),
                                 tr.empty() ? nullptr : tr.data(), nullptr));
  }
};

enum class AddMode { replace, increment };

struct ShallowWaterModel;

// A tendency-term member of the model (shallow_water_model.hpp:19-29): its
// m_enabled reads and switches the term through the library, so
// `model.m_pv_flux_edge.m_enabled = false;` works as in the reference.
struct TermSwitch {
  const ShallowWaterModel *m_model;
  int m_term;
  operator bool() const;
  TermSwitch &operator=(bool on);
  TermSwitch(const ShallowWaterModel *model, int term)
      : m_model(model), m_term(term) {}
  TermSwitch(const TermSwitch &) = delete;
};
struct TendencyTerm {
  TermSwitch m_enabled;
  TendencyTerm(const ShallowWaterModel *model, int term)
      : m_enabled(model, term) {}
};

// Read-only view of the model's auxiliary state (the reference's
// ShallowWaterAuxiliaryState, shallow_water_auxstate.hpp, with its member
// groups): device views of the intermediates of the last auxiliary
// computation, which compute() or any tendency evaluation or step leaves.
// The GPU path keeps the mean thickness once (m_mean_h_edge and
// m_flux_h_edge, equal in the reference, view the same array) and the two
// vorticity terms summed: m_pv_vertex = norm_rvort_vertex +
// norm_pvort_vertex, m_pv_edge = 2 (norm_rvort_edge + norm_pvort_edge).
// A view the model's configuration does not compute is empty (null data).
struct ShallowWaterAuxiliaryState {
  swg_model m_model = nullptr;
  struct {
    RealConst2d m_mean_h_edge, m_flux_h_edge;
  } m_thickness_aux;
  struct {
    RealConst2d m_rvort_vertex, m_pv_vertex, m_pv_edge;
  } m_vorticity_aux;
  struct {
    RealConst2d m_ke_cell, m_vel_div_cell;
  } m_kinetic_aux;
  struct {
    RealConst3d m_norm_tr_cell;
  } m_tracer_aux;
  // shallow_water_auxstate.cpp:12-50; f_vertex is the model's m_f_vertex
  void compute(RealConst2d h_cell, RealConst2d vn_edge, RealConst3d tr_cell,
               RealConst1d /*f_vertex*/, const void * /*mesh*/ = nullptr) const {
    swg_check(swg_model_compute_aux(m_model, h_cell.data(), vn_edge.data(),
                                    tr_cell.data(), nullptr));
  }
};

struct ShallowWaterModel {
  ShallowWaterParams m_params;
  MPASMesh *m_mesh;
  swg_model m_handle = nullptr;

  TendencyTerm m_thickness_hadv_cell{this, SWG_TERM_THICKNESS_HADV};
  TendencyTerm m_pv_flux_edge{this, SWG_TERM_PV_FLUX};
  TendencyTerm m_ke_grad_edge{this, SWG_TERM_KE_GRAD};
  TendencyTerm m_ssh_grad_edge{this, SWG_TERM_SSH_GRAD};
  TendencyTerm m_vel_diff_edge{this, SWG_TERM_VEL_DIFF};
  TendencyTerm m_vel_hyperdiff_edge{this, SWG_TERM_VEL_HYPERDIFF};
  TendencyTerm m_tracer_hadv_cell{this, SWG_TERM_TRACER_HADV};
  TendencyTerm m_tracer_diff_cell{this, SWG_TERM_TRACER_DIFF};
  TendencyTerm m_tracer_hyperdiff_cell{this, SWG_TERM_TRACER_HYPERDIFF};
  // Coriolis parameter per vertex (shallow_water_model.hpp:32), f0 after
  // construction; a user kernel may write it, later evaluations read it
  Real1d m_f_vertex;
  // the auxiliary state of the last evaluation (shallow_water_model.hpp:18)
  ShallowWaterAuxiliaryState m_aux_state;

  // `options`: the linear variant or the opt-in bottom drag
  // (swg_model_options in swgpu.h); the default is the reference's model,
  // which ignores m_drag_coeff.
  ShallowWaterModel(MPASMesh *mesh, const ShallowWaterParams &params,
                    const swg_model_options &options = swg_model_options{})
      : m_params(params), m_mesh(mesh) {
    swg_params p{params.m_f0,         params.m_grav,       params.m_drag_coeff,
                 params.m_visc_del2,  params.m_visc_del4,  params.m_eddy_diff2,
                 params.m_eddy_diff4, params.m_ntracers,
                 params.m_disable_h_tendency ? 1 : 0,
                 params.m_disable_vn_tendency ? 1 : 0};
    swg_check(swg_model_create_ex(mesh->m_handle, &p, &options, &m_handle));
    const double *fv = nullptr;
    long long nfv = 0;
    swg_check(swg_model_aux(m_handle, "f_vertex", &fv, &nfv));
    m_f_vertex.m_data = const_cast<double *>(fv);
    m_f_vertex.m_ext[0] = size_t(nfv);
    bind_aux_state();
    // The hook is registered here, where the dynamic type is not known yet.
    // settle_hook() drops it without any GPU work for the library's own
    // model classes (steppers, compute_tendency and resolve_hook call it);
    // for a user's derived class it stays until the base no-op runs once
    // (an override keeps the unfused, hooked sequence).
    swg_check(swg_model_set_forcing(m_handle, &ShallowWaterModel::trampoline,
                                    this));
  }
  ShallowWaterModel(const ShallowWaterModel &) = delete;
  ShallowWaterModel &operator=(const ShallowWaterModel &) = delete;
  virtual ~ShallowWaterModel() { swg_model_destroy(m_handle); }

  // shallow_water_model.hpp:42-44 (h_tend_cell, vn_tend_edge, h_cell,
  // vn_edge, t); the base adds nothing
  virtual void additional_tendency(Real2d /*h_tend_cell*/,
                                   Real2d /*vn_tend_edge*/,
                                   RealConst2d /*h_cell*/,
                                   RealConst2d /*vn_edge*/,
                                   Real /*t*/) const {
    m_default_hook = true;
  }

  void compute_tendency(const ShallowWaterState &tend,
                        const ShallowWaterState &state, Real t,
                        AddMode add_mode = AddMode::replace) const {
    settle_hook();
    const int rc = swg_compute_tendency(
        m_handle, tend.handle(), state.handle(), t,
        add_mode == AddMode::replace ? SWG_ADD_REPLACE : SWG_ADD_INCREMENT,
        nullptr);
    rethrow_hook_error();
    swg_check(rc);
  }

  // shallow_water_model.hpp:36-41: one field's tendency from the auxiliary
  // state of the last evaluation (m_aux_state) and the given views; the
  // tracer tendency reads the normalised tracers of the auxiliary state
  // (tr_cell is not read, and no h is given, as in the reference)
  void compute_h_tendency(Real2d h_tend_cell, RealConst2d h_cell,
                          RealConst2d vn_edge, AddMode add_mode) const {
    swg_check(swg_compute_h_tendency(m_handle, h_tend_cell.data(),
                                     h_cell.data(), vn_edge.data(),
                                     mode(add_mode), nullptr));
  }
  void compute_vn_tendency(Real2d vn_tend_edge, RealConst2d h_cell,
                           RealConst2d vn_edge, AddMode add_mode) const {
    swg_check(swg_compute_vn_tendency(m_handle, vn_tend_edge.data(),
                                      h_cell.data(), vn_edge.data(),
                                      mode(add_mode), nullptr));
  }
  void compute_tr_tendency(Real3d tr_tend_cell, RealConst3d tr_cell,
                           RealConst2d vn_edge, AddMode add_mode) const {
    swg_check(swg_compute_tr_tendency(m_handle, tr_tend_cell.data(),
                                      tr_cell.data(), vn_edge.data(),
                                      mode(add_mode), nullptr));
  }

  // Drops the hook registered at construction when additional_tendency
  // cannot be overridden: the object is exactly a ShallowWaterModel or a
  // LinearShallowWaterModel (a user's derived class may override it and
  // keeps the hook).  Costs no GPU work; the steppers, the tendency call and
  // resolve_hook() run it first.
  void settle_hook() const;

  // An exception thrown by an additional_tendency override does not cross
  // the C ABI: the hook's trampoline keeps it, and the call that ran the
  // hook (compute_tendency, do_step, do_steps) rethrows it after the library
  // returns.  The state is then unspecified, as after an exception in the
  // reference's step.
  void rethrow_hook_error() const {
    if (m_hook_error) {
      std::exception_ptr e = m_hook_error;
      m_hook_error = nullptr;
      std::rethrow_exception(e);
    }
  }

  // Settles whether additional_tendency is overridden: one tendency
  // evaluation on a scratch state (h = vn = 1) runs the hook once; the base
  // no-op then unregisters itself.  The ensemble and adjoint classes call it
  // because the library refuses models that still carry a hook.
  void resolve_hook() const {
    settle_hook();
    if (m_default_hook)
      return;
    ShallowWaterState tend(m_mesh, m_params), state(m_mesh, m_params);
    swg_check(swg_state_fill(state.handle(), 1.0, nullptr));
    compute_tendency(tend, state, 0.0);
    fence();
  }

private:
  mutable bool m_default_hook = false;
  mutable std::exception_ptr m_hook_error; // the first one since the call

  static int mode(AddMode m) {
    return m == AddMode::replace ? SWG_ADD_REPLACE : SWG_ADD_INCREMENT;
  }
  // m_aux_state's views of the model's intermediate arrays
  void bind_aux_state() {
    ShallowWaterAuxiliaryState &a = m_aux_state;
    a.m_model = m_handle;
    const MPASMesh *me = m_mesh;
    auto bind2 = [&](const char *name, RealConst2d &v, Int rows) {
      const double *p = nullptr;
      long long n = 0;
      if (swg_model_aux(m_handle, name, &p, &n) != SWG_OK)
        return; // not computed by this configuration: an empty view
      v.m_data = p;
      v.m_ext[0] = rows;
      v.m_ext[1] = me->m_nlayers;
    };
    bind2("mean_h_edge", a.m_thickness_aux.m_mean_h_edge, me->m_nedges);
    a.m_thickness_aux.m_flux_h_edge = a.m_thickness_aux.m_mean_h_edge;
    bind2("rvort_vertex", a.m_vorticity_aux.m_rvort_vertex, me->m_nvertices);
    bind2("q_vertex", a.m_vorticity_aux.m_pv_vertex, me->m_nvertices);
    bind2("pv_edge", a.m_vorticity_aux.m_pv_edge, me->m_nedges);
    bind2("ke_cell", a.m_kinetic_aux.m_ke_cell, me->m_ncells);
    bind2("vel_div_cell", a.m_kinetic_aux.m_vel_div_cell, me->m_ncells);
    const double *p = nullptr;
    long long n = 0;
    if (m_params.m_ntracers > 0 &&
        swg_model_aux(m_handle, "norm_tr_cell", &p, &n) == SWG_OK) {
      RealConst3d &t = a.m_tracer_aux.m_norm_tr_cell;
      t.m_data = p;
      t.m_ext[0] = m_params.m_ntracers;
      t.m_ext[1] = me->m_ncells;
      t.m_ext[2] = me->m_nlayers;
    }
  }

  static void trampoline(void *user, double *h_tend, double *vn_tend,
                         const double *h, const double *vn, double t,
                         void *) {
    auto *self = static_cast<ShallowWaterModel *>(user);
    if (self->m_hook_error) // the rest of a failed call runs without it
      return;
    const MPASMesh *m = self->m_mesh;
    Real2d ht, vt;
    RealConst2d hc, vc;
    ht.m_data = h_tend;
    vt.m_data = vn_tend;
    hc.m_data = h;
    vc.m_data = vn;
    ht.m_ext[0] = hc.m_ext[0] = m->m_ncells;
    vt.m_ext[0] = vc.m_ext[0] = m->m_nedges;
    ht.m_ext[1] = hc.m_ext[1] = vt.m_ext[1] = vc.m_ext[1] = m->m_nlayers;
    try {
      self->additional_tendency(ht, vt, hc, vc, t);
    } catch (...) {
      if (!self->m_hook_error)
        self->m_hook_error = std::current_exception();
      return;
    }
    if (self->m_default_hook)
      swg_model_set_forcing(self->m_handle, nullptr, nullptr);
  }
};

inline TermSwitch::operator bool() const {
  int on = 0;
  swg_check(swg_model_term_enabled(m_model->m_handle, m_term, &on));
  return on != 0;
}
inline TermSwitch &TermSwitch::operator=(bool on) {
  swg_check(swg_model_set_term_enabled(m_model->m_handle, m_term, on ? 1 : 0));
  return *this;
}

// LinearShallowWaterModel and its parameters
// (shallow_water_hierarchical.cpp:676-775): h_t = -h0 div(vn),
// vn_t = f0 sum_j w_j vn_j - g grad h; no tracers, no dissipation.
struct LinearShallowWaterParams : ShallowWaterParams {
  Real m_h0 = 1000;
};

struct LinearShallowWaterModel : ShallowWaterModel {
  LinearShallowWaterModel(MPASMesh *mesh, const LinearShallowWaterParams &params)
      : ShallowWaterModel(mesh, params, swg_model_options{1, params.m_h0, 0}),
        m_h0(params.m_h0) {}
  Real m_h0;
};

inline void ShallowWaterModel::settle_hook() const {
  if (m_default_hook || (typeid(*this) != typeid(ShallowWaterModel) &&
                         typeid(*this) != typeid(LinearShallowWaterModel)))
    return;
  m_default_hook = true;
  swg_check(swg_model_set_forcing(m_handle, nullptr, nullptr));
}

// --------------------------------------------------------------- steppers --

struct TimeStepper {
  ShallowWaterModel *m_shallow_water;
  swg_stepper m_handle = nullptr;
  virtual void do_step(Real t, Real dt,
                       const ShallowWaterState &state) const {
    const int rc = swg_step(m_handle, state.handle(), t, dt, 1, 1, nullptr);
    m_shallow_water->rethrow_hook_error();
    swg_check(rc);
  }
  // nsteps consecutive do_step calls from t0 in one library call
  void do_steps(Real t0, Real dt, const ShallowWaterState &state,
                Int nsteps) const {
    const int rc =
        swg_step(m_handle, state.handle(), t0, dt, nsteps, 1, nullptr);
    m_shallow_water->rethrow_hook_error();
    swg_check(rc);
  }
  TimeStepper(ShallowWaterModel &shallow_water, int kind, int nstages)
      : m_shallow_water(&shallow_water) {
    shallow_water.settle_hook(); // the model is fully constructed here
    swg_check(swg_stepper_create(shallow_water.m_handle, kind, nstages,
                                 &m_handle));
  }
  TimeStepper(const TimeStepper &) = delete;
  TimeStepper &operator=(const TimeStepper &) = delete;
  virtual ~TimeStepper() { swg_stepper_destroy(m_handle); }
};

struct LSRKStepper : TimeStepper {
  Int m_nstages;
  LSRKStepper(ShallowWaterModel &shallow_water, Int nstages = 5)
      : TimeStepper(shallow_water, SWG_STEPPER_LSRK, nstages),
        m_nstages(nstages) {}
};

struct RK4Stepper : TimeStepper {
  static constexpr Int nstages = 4;
  explicit RK4Stepper(ShallowWaterModel &shallow_water)
      : TimeStepper(shallow_water, SWG_STEPPER_RK4, 4) {}
};

// A state kept in host arrays (h [C][K], vn [E][K], tr [T][C][K]) advanced
// in place, level chunk by level chunk, with each chunk's copies overlapping
// the other chunks' compute (swg_host_stepper_*).  Bitwise equal to upload +
// do_steps + download.  The model must have no additional_tendency override
// and must outlive the stepper.  No counterpart in the reference.
struct HostStepper {
  swg_host_stepper m_handle = nullptr;
  HostStepper(ShallowWaterModel &shallow_water, bool rk4 = false,
              Int nstages = 5, Int level_chunk = 0) {
    shallow_water.resolve_hook();
    swg_check(swg_host_stepper_create(
        shallow_water.m_handle, rk4 ? SWG_STEPPER_RK4 : SWG_STEPPER_LSRK,
        rk4 ? 4 : nstages, level_chunk, &m_handle));
  }
  HostStepper(const HostStepper &) = delete;
  HostStepper &operator=(const HostStepper &) = delete;
  ~HostStepper() { swg_host_stepper_destroy(m_handle); }
  void do_steps(Real t0, Real dt, double *h, double *vn, double *tr,
                Int nsteps) const {
    swg_check(swg_host_step(m_handle, h, vn, tr, t0, dt, nsteps, nullptr));
  }
};

// ----------------------------------------------- ensembles and gradients --
// Beside the plain solver; no counterpart in the reference.

// Many independent members (own mesh size, levels and tracers) advanced
// together: one persistent kernel, or one launch per pass, per RK stage
// (swg_batch_*).  Members must have distinct models and states, and those
// must outlive the stepper (it keeps their handles).
struct EnsembleStepper {
  swg_batch m_handle = nullptr;
  EnsembleStepper(const std::vector<ShallowWaterModel *> &models,
                  const std::vector<const ShallowWaterState *> &states,
                  bool rk4 = true, Int nstages = 4) {
    std::vector<swg_model> mh;
    std::vector<swg_state> sh;
    for (auto *m : models) {
      m->resolve_hook();
      mh.push_back(m->m_handle);
    }
    for (auto *s : states)
      sh.push_back(s->handle());
    if (mh.size() != sh.size())
      throw std::runtime_error("EnsembleStepper: models and states differ in number");
    swg_check(swg_batch_create(int(mh.size()), mh.data(), sh.data(),
                               rk4 ? SWG_STEPPER_RK4 : SWG_STEPPER_LSRK,
                               rk4 ? 4 : nstages, &m_handle));
  }
  EnsembleStepper(const EnsembleStepper &) = delete;
  EnsembleStepper &operator=(const EnsembleStepper &) = delete;
  ~EnsembleStepper() { swg_batch_destroy(m_handle); }
  // times every launch configuration on these members (advancing them) and
  // keeps the fastest; returns its index
  int autotune(Real dt, int reps = 2, double *ms_per_step = nullptr) {
    int best = 0;
    double ms = 0;
    swg_check(swg_batch_autotune(m_handle, dt, reps, nullptr, &best, &ms));
    if (ms_per_step)
      *ms_per_step = ms;
    return best;
  }
  void do_steps(Real t0, Real dt, Int nsteps) const {
    swg_check(swg_batch_step(m_handle, t0, dt, nsteps, 1, nullptr));
    swg_check(swg_batch_check(m_handle, nullptr));
  }
};

// Gradient of a loss of the state after nsteps RK4 steps with respect to the
// initial state (and the del2 viscosity), by the hand-written adjoint with
// binomial checkpointing over `nsnapshots` states (swg_adjoint_*):
//   adj.forward(x0, t0, dt, n, xN);  lambda <- dL/dxN;  adj.backward(lambda);
//   lambda now holds dL/dx0.
struct CheckpointedAdjoint {
  swg_adjoint m_handle = nullptr;
  // kind: SWG_STEPPER_RK4, or SWG_STEPPER_LSRK with nstages 5 or 1
  explicit CheckpointedAdjoint(ShallowWaterModel &model, Int nsnapshots = 32,
                               int kind = SWG_STEPPER_RK4, Int nstages = 4) {
    model.resolve_hook();
    swg_check(swg_adjoint_create_stepper(model.m_handle, nsnapshots, kind,
                                         nstages, &m_handle));
  }
  CheckpointedAdjoint(const CheckpointedAdjoint &) = delete;
  CheckpointedAdjoint &operator=(const CheckpointedAdjoint &) = delete;
  ~CheckpointedAdjoint() { swg_adjoint_destroy(m_handle); }
  void forward(const ShallowWaterState &x0, Real t0, Real dt, Int nsteps,
               const ShallowWaterState &xN) {
    swg_check(swg_adj_forward(m_handle, x0.handle(), t0, dt, nsteps,
                              xN.handle(), nullptr));
  }
  void backward(const ShallowWaterState &lambda) {
    swg_check(swg_adj_backward(m_handle, lambda.handle(), nullptr));
  }
  // dx <- J dx over nsteps steps from x0 (tangent-linear model)
  void tlm_apply(const ShallowWaterState &x0, const ShallowWaterState &dx,
                 Real t0, Real dt, Int nsteps) {
    swg_check(swg_tlm_apply(m_handle, x0.handle(), dx.handle(), t0, dt,
                            nsteps, nullptr));
  }
  // dL/d(viscosity) of the last backward: per edge and per cell
  void grad_visc(std::vector<Real> &per_edge, std::vector<Real> &per_cell,
                 const MPASMesh &mesh) {
    per_edge.resize(mesh.m_nedges);
    per_cell.resize(mesh.m_ncells);
    swg_check(swg_adj_grad_visc(m_handle, per_edge.data(), per_cell.data(),
                                nullptr));
  }
  long long plain_steps() const {
    long long p = 0, t = 0;
    swg_check(swg_adj_info(m_handle, &p, &t));
    return p;
  }
  // steps of the last sweep pair taped as taped advances (the last step of
  // a re-advance, kept in the second tape for the next reversal)
  long long taped_advances() const {
    long long p = 0, t = 0, a = 0;
    swg_check(swg_adj_info_ex(m_handle, &p, &t, &a));
    return a;
  }
};

// Many members' gradients at once (swg_adj_ensemble_*): members with the
// same schedule run in lockstep, every action one launch per pass over all
// of them.  Each member's result equals its own CheckpointedAdjoint's bit
// for bit; the adjoints stay owned by the caller and must outlive this.
//   CheckpointedAdjointEnsemble ens({&a0, &a1, ...});
//   ens.forward({&x0_0, ...}, t0, dt, n, {&xN_0, ...});
//   ens.backward({&lambda_0, ...});
struct CheckpointedAdjointEnsemble {
  swg_adj_ensemble m_handle = nullptr;
  Int m_size = 0;
  explicit CheckpointedAdjointEnsemble(
      const std::vector<CheckpointedAdjoint *> &adjoints) {
    std::vector<swg_adjoint> h;
    for (CheckpointedAdjoint *a : adjoints)
      h.push_back(a->m_handle);
    m_size = Int(h.size());
    swg_check(swg_adj_ensemble_create(m_size, h.data(), &m_handle));
  }
  CheckpointedAdjointEnsemble(const CheckpointedAdjointEnsemble &) = delete;
  CheckpointedAdjointEnsemble &
  operator=(const CheckpointedAdjointEnsemble &) = delete;
  ~CheckpointedAdjointEnsemble() { swg_adj_ensemble_destroy(m_handle); }
  void forward(const std::vector<const ShallowWaterState *> &x0, Real t0,
               Real dt, Int nsteps,
               const std::vector<const ShallowWaterState *> &xN) {
    const std::vector<swg_state> a = handles(x0), b = handles(xN);
    swg_check(swg_adj_ensemble_forward(m_handle, a.data(), t0, dt, nsteps,
                                       b.data(), nullptr));
  }
  void backward(const std::vector<const ShallowWaterState *> &lambda) {
    const std::vector<swg_state> l = handles(lambda);
    swg_check(swg_adj_ensemble_backward(m_handle, l.data(), nullptr));
  }
  // lockstep groups, and each member's group
  Int groups(std::vector<int> *group_of = nullptr) const {
    int n = 0;
    if (group_of)
      group_of->resize(m_size);
    swg_check(swg_adj_ensemble_groups(m_handle, &n,
                                      group_of ? group_of->data() : nullptr));
    return n;
  }

private:
  std::vector<swg_state>
  handles(const std::vector<const ShallowWaterState *> &s) const {
    if (Int(s.size()) != m_size)
      throw std::runtime_error(
          "CheckpointedAdjointEnsemble: one state per member");
    std::vector<swg_state> h;
    for (const ShallowWaterState *x : s)
      h.push_back(x->handle());
    return h;
  }
};

// ------------------------------------------------------------ diagnostics --

inline Real energy_integral(const ShallowWaterState &state,
                            const ShallowWaterModel &model) {
  Real out;
  swg_check(swg_diag_energy(model.m_handle, state.handle(), &out, nullptr));
  return out;
}
inline Real mass_integral(const ShallowWaterState &state,
                          const ShallowWaterModel &model) {
  Real out;
  swg_check(swg_diag_mass(model.m_handle, state.handle(), &out, nullptr));
  return out;
}
inline Real circulation_integral(const ShallowWaterState &state,
                                 const ShallowWaterModel &model) {
  Real out;
  swg_check(
      swg_diag_circulation(model.m_handle, state.handle(), &out, nullptr));
  return out;
}

} // namespace omega
