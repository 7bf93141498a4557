// Internal declarations of the GB300 shallow-water library (not installed).
#pragma once

#include "../../include/swgpu.h"

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <string>
#include <vector>

namespace swg {

// Records the calling thread's error message and returns `code`.
int fail(int code, const std::string &msg);
// Maps a CUDA error to SWG_ERR_CUDA (or SWG_ERR_OOM) with context.
int cuda_fail(cudaError_t err, const char *what);

// The C ABI throws nothing: every entry point is a function-try-block whose
// handler turns a host-side exception (in practice std::bad_alloc from a
// container) into a status: SWG_ERR_OOM for a failed allocation,
// SWG_ERR_ARG otherwise.  Called only from a handler.
int abi_exception(const char *entry) noexcept;
#define SWG_ABI_CATCH(entry)                                                   \
  catch (...) {                                                                \
    return swg::abi_exception(entry);                                          \
  }

// Return the status of a call that failed (anything but SWG_OK).
#define TRY(x)                                                                 \
  do {                                                                         \
    int rc_ = (x);                                                             \
    if (rc_ != SWG_OK)                                                         \
      return rc_;                                                              \
  } while (0)

int build_planar_hex(int nx, int ny, double dc, swg_hex_tables *t,
                     double *period_x, double *period_y);

extern std::atomic<long long> g_launches;

constexpr int MAXE = 6; // edges per cell (MPASMesh::maxedges)

// Device views of the K-independent tables derived from the MPAS tables.
// Per-cell slots beyond nedges_on_cell are padded with coefficient 0 and a
// valid index, so kernels loop a fixed MAXE times without branches.
struct MeshView {
  int ncells, nedges, nvertices, nlayers;
  int ne;           // compacted edges-on-edge slots per edge (8 or 10)
  int dv4_differs;  // some edge has dv < dc/4 (the del4 Laplacian differs)
  // vertices [V][3]
  const int *ev;      // edges_on_vertex
  const int *cv;      // cells_on_vertex
  const double *cvr;  // dc * (1/area_triangle) * edge_sign_on_vertex
  const double *kvh;  // kiteareas * (1/area_triangle)
  // cells [C][6]
  const int *ec;      // edges_on_cell
  const int *nbc;     // cell across edge j
  const double *ccd;  // (1/area_cell) * dv * edge_sign_on_cell
  const double *cke;  // (1/area_cell) * dv * dc * 0.25
  const double *ckq;  // (1/area_cell) * dv * (1/dc)    (>= 0)
  const double *ccdh; // -0.5 * ccd
  // edges
  const int *ce;      // cells_on_edge [E][2]
  const int *ve;      // vertices_on_edge [E][2]
  const double *inv_dc, *inv_dv, *inv_dv4; // [E]
  const int *eoe;     // nonzero-weight edges_on_edge [E][ne]
  const double *woe;  // their weights / 4 [E][ne]
  const double *scale2, *scale4; // [E]
  const double *mask; // edge_mask [E][K], nullptr when all ones
  // diagnostics only
  const double *area_cell_d; // [C]
  const double *area_tri_d;  // [V]
  const double *dcs_v;       // [V][3] dc * edge_sign_on_vertex
  const int *maxlev_c;       // [C] levels summed per cell, nullptr = nlayers
  const int *maxlev_v;       // [V] levels summed per vertex, nullptr = nlayers
};

// Parameters and parameter-scaled coefficient tables of one model.
struct ModelView {
  double grav;
  const double *f_vertex; // [V]
  const double *gidc;     // [E] grav / dc
  const double *c2e;      // [E] visc_del2 * scale2
  const double *c4e;      // [E] -visc_del4 * scale4
  // [E] c4e / dc and -c4e / dv: the del4 tendency's outer Laplacian with
  // the coefficient folded in (used without an edge mask; nullptr = unused)
  const double *c4i, *c4v;
  const double *kd2;      // [C][6] eddy_diff2 * scale2 * ckq
  const double *r4;       // [C][6] -eddy_diff4 * scale4 * ckq
  const double *r4sum;    // [C] sum of r4
  // [C] eddy_diff2 * s - r4sum when mesh_scaling_del2 is s on every edge,
  // else nullptr.  The tracer del2 term is then eddy_diff2 * s times the
  // thickness-weighted Laplacian the del4 term already computes, so it
  // folds into the centre weight of the del4 stencil.
  const double *r4f;
  int ntracers;
  int vel_del2, vel_del4, tr_del2, tr_del4, do_h, do_vn;
  // LinearShallowWaterModel (mean thickness h0; f4 = 4 f0, the Coriolis
  // factor for the weights/4 table), and the optional bottom drag
  int linear, drag;
  int drag_level; // the level of the model's arrays that carries the drag
  double h0, f4, drag_coeff;
  // tendency terms switched off after create (the reference's m_enabled
  // members); zero = on, so zero-initialised views keep every term
  int off_hadv, off_pv, off_ke, off_ssh, off_tr_hadv;
};

// Forward-mode dual number (value, tangent) of the tangent-linear model;
// its device arithmetic is in swg_device.cuh.
struct Dual {
  double v, d;
};

// Intermediate fields of one tendency evaluation (device), templated on
// the value type: double, or Dual (value + tangent) for the tangent-linear
// model.
template <class T> struct AuxViewT {
  T *q, *zeta, *z4;              // [V][K]
  T *div, *ke, *d4;              // [C][K]
  T *ntr, *lap;                  // [T][C][K]
  T *F, *G, *Q, *mh, *u2, *d2u, *d2u4; // [E][K]
  // written only when set (the adjoint's tape): 1/h_vertex [V][K], 1/h
  // [C][K] and the PV-flux sum S1 = sum_j w_j F_j [E][K]
  T *rhv, *rh, *S1;
};
using AuxView = AuxViewT<double>;

enum EpiMode {
  EPI_REPLACE = 0,   // tend = x
  EPI_INCREMENT = 1, // tend += x
  EPI_LSRK = 2,      // t = a*tend + x; tend = t; state += dtb*t
  EPI_RK4_FIRST = 3, // acc = old + dtb*x; out = old + dta*x
  EPI_RK4_MID = 4,   // acc += dtb*x;      out = old + dta*x
  EPI_RK4_LAST = 5,  // out = acc + dtb*x
  EPI_LSRK_TEND = 6, // t = a*tend + x; tend = t (state updated afterwards)
};

template <class T> struct FieldIOT {
  T *tend;      // REPLACE / INCREMENT / LSRK
  const T *old; // RK4 first & mid: state at the start of the step
  T *acc;       // RK4: accumulator
  T *out;       // LSRK: state; RK4: next stage input or final state
};
using FieldIO = FieldIOT<double>;

struct Epilogue {
  int mode;
  double a, dtb, dta;
};

template <class T> struct StageArgsT {
  const T *h, *vn, *tr; // stage input state
  FieldIOT<T> fh, fvn, ftr;
  Epilogue ep;
};
using StageArgs = StageArgsT<double>;

// NVTX range (header-only NVTX3; no cost without a tool attached), named
// after the reference's Caliper regions (shallow_water_model.cpp:317-346:
// auxstate, tendencies, h_tendency, vn_tendency, tr_tendency;
// benchmark.cpp:154,166: time_integration) so timelines read alike.
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

// A second stream and two events owned by a model: independent passes of
// one evaluation run as a fork/join pair on it (inside captured graphs they
// become parallel branches), so that one pass fills the other's last wave.
struct Fork {
  cudaStream_t side = nullptr;
  cudaEvent_t go = nullptr, done = nullptr;
};
int fork_create(Fork &f);
void fork_destroy(Fork &f);
// runs main_fn on st and side_fn on the fork's stream concurrently (in that
// order on st when fk is null)
template <class A, class B>
void fork_join(const Fork *fk, cudaStream_t st, A main_fn, B side_fn) {
  if (!fk || !fk->side) {
    main_fn(st);
    side_fn(st);
    return;
  }
  cudaEventRecord(fk->go, st);
  cudaStreamWaitEvent(fk->side, fk->go, 0);
  side_fn(fk->side);
  cudaEventRecord(fk->done, fk->side);
  main_fn(st);
  cudaStreamWaitEvent(st, fk->done, 0);
}

// fk (optional): run the independent passes concurrently
void launch_tendency(const MeshView &m, const ModelView &p, const AuxView &a,
                     const StageArgs &s, cudaStream_t st,
                     const Fork *fk = nullptr);
// the same six passes on dual numbers (tangent-linear model)
void launch_tendency_dual(const MeshView &m, const ModelView &p,
                          const AuxViewT<Dual> &a, const StageArgsT<Dual> &s,
                          cudaStream_t st);
// only the four auxiliary passes (intermediates of the state h, vn, tr)
void launch_aux(const MeshView &m, const ModelView &p, const AuxView &a,
                const double *h, const double *vn, const double *tr,
                cudaStream_t st, const Fork *fk = nullptr);
// one field of a tendency from the last auxiliary state in `a` and the
// caller's h / vn (the reference's compute_h_tendency, compute_vn_tendency,
// compute_tr_tendency): field 0 h, 1 vn, 2 tracers; mode EPI_REPLACE or
// EPI_INCREMENT.  Rewrites the thickness flux F (and G) of `a`.
void launch_field_tendency(const MeshView &m, const ModelView &p,
                           const AuxView &a, int field, const double *h,
                           const double *vn, double *tend, int mode,
                           cudaStream_t st);
void launch_axpby(double *y, const double *x, const double *z, double alpha,
                  double beta, long long n, int kind, cudaStream_t st);
// opt-in per-kernel CUDA-event timing (swg_profile_enable)
bool profiling_enabled();
// while alive, launches of the calling thread are not timed (no events are
// created for them) even with profiling on
struct ProfileOff {
  ProfileOff();
  ~ProfileOff();
  ProfileOff(const ProfileOff &) = delete;
  ProfileOff &operator=(const ProfileOff &) = delete;
};
int profile_enable(int on);
int profile_read(int max_kernels, char *names, double *total_ms,
                 long long *launches, int *count);
int reduce_diag(int which, const MeshView &m, const ModelView &p,
                const double *h, const double *vn, double *partials,
                int npart, double *out, cudaStream_t st);

} // namespace swg

// ------------------------------------------------------------- handles ---

struct swg_mesh_s {
  int ncells, nedges, nvertices, nlayers;
  swg::MeshView view;
  std::vector<void *> allocs;
  // host copies of the per-edge scaling (the model scales them)
  std::vector<double> scale2_h, scale4_h, ckq_h, inv_dc_h;
  bool scale2_uniform = false; // mesh_scaling_del2 the same on every edge
  std::vector<int> ec_h, nec_h; // edges_on_cell (padded), nedges_on_cell
  // host copies of the derived tables (the adjoint builds transposes)
  std::vector<int> ev_h, cv_h, nbc_h, ce_h, ve_h, eoe_h;
  std::vector<double> cvr_h, kvh_h, ccd_h, cke_h, ccdh_h, inv_dv_h, woe_h;
  std::vector<double> inv_dv4_h; // 1 / max(dv, dc / 4)
};

struct swg_state_s {
  swg_mesh mesh;
  int ntracers;
  double *h, *vn, *tr;
  void *block;
  // creation number, never reused: identifies the state in cached graphs
  // (a handle address can be reused after destroy, with other device memory)
  unsigned long long serial;
};

struct swg_model_s {
  swg_mesh mesh;
  swg_params params;
  swg::ModelView view;
  swg::AuxView aux;
  std::vector<void *> allocs;
  double *partials; // diagnostic partial sums
  swg_forcing_fn forcing;
  void *forcing_user;
  swg::Fork fork;
  // bumped when a term is switched (captured step graphs hold the view)
  unsigned long long version;
  int terms_switched; // some term differs from what create enabled
};

struct swg_stepper_s {
  swg_model model;
  int kind, nstages;
  std::vector<double> rka, rkb, rkc;
  swg_state tend, acc, p0, p1, old;
  cudaGraphExec_t graph;       // one captured step (fused path)
  unsigned long long graph_serial; // the state the graph was captured for
  unsigned long long graph_version; // and the model's term version
  double graph_dt;
  long long graph_launches;    // kernels per captured step
};
