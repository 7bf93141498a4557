/*
 * swgpu.h - C ABI of the GB300 shallow-water solver (omega_playground_gb300).
 *
 * The solver replaces the Kokkos device path of mwarusz/omega_playground:
 * its mesh tables, model state, tendency terms and time steppers.  The C++
 * classes in omega_playground_gb300/cxx/omega_gpu.hpp keep the reference's
 * class names and signatures and call these functions; other hosts (Python
 * ctypes, Fortran, ...) can bind them directly.  All reference citations are
 * paths inside the omega_playground checkout.
 *
 * Conventions
 *  - Every function returns an int status (SWG_OK = 0), except the
 *    accessors swg_last_error, swg_version, swg_kernel_launches and
 *    swg_checkpoint_cost (-1 on error); nothing throws or aborts across the
 *    ABI (a host allocation that fails inside a call is SWG_ERR_OOM).
 *    swg_last_error() gives the calling thread's message for the last
 *    failed call.
 *  - Arrays are FP64 [entity][k] row-major with the level index k contiguous;
 *    tracers are [l][cell][k]; connectivity is int32.  "host" pointers are
 *    CPU memory, "device" pointers are CUDA global memory on the current
 *    device.
 *  - Handles are thread-confined.  Compute calls take a cudaStream_t (passed
 *    as void*, NULL = legacy default stream) and are asynchronous on it;
 *    the calls that block the host are swg_state_download, swg_diag_*,
 *    swg_sync, swg_host_step, swg_batch_check, swg_batch_autotune,
 *    swg_adj_grad_visc and swg_profile_read.
 *  - A model's intermediate fields are shared by every call on it (as the
 *    reference's model holds one auxiliary state), so calls on one model, or
 *    on steppers and adjoints built on it, must be ordered: one stream, or
 *    events between streams.  Different models run concurrently.
 *  - Connectivity is validated on the host at swg_mesh_create: every index
 *    is checked against its table's range before any kernel can read it.
 */
#ifndef SWGPU_H
#define SWGPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define SWG_OK 0
#define SWG_ERR_ARG 1        /* bad argument or inconsistent sizes */
#define SWG_ERR_OOM 2        /* device or host allocation failed */
#define SWG_ERR_CUDA 3       /* a CUDA runtime call failed */
#define SWG_ERR_TIMEOUT 4    /* a bounded device wait expired */
#define SWG_ERR_BUDGET 5     /* checkpoint budget too small */
#define SWG_ERR_STATE 6      /* handle used in the wrong state */

#define SWG_ADD_REPLACE 0    /* AddMode::replace   (shallow_water_model.hpp:11) */
#define SWG_ADD_INCREMENT 1  /* AddMode::increment (shallow_water_model.hpp:11) */

#define SWG_STEPPER_RK4 0    /* RK4Stepper  (time_stepper.hpp:27-38) */
#define SWG_STEPPER_LSRK 1   /* LSRKStepper (time_stepper.hpp:16-25) */

typedef struct swg_mesh_s *swg_mesh;
typedef struct swg_state_s *swg_state;
typedef struct swg_model_s *swg_model;
typedef struct swg_stepper_s *swg_stepper;
typedef struct swg_batch_s *swg_batch;
typedef struct swg_adjoint_s *swg_adjoint;
typedef struct swg_host_stepper_s *swg_host_stepper;
typedef struct swg_adj_ensemble_s *swg_adj_ensemble;

/* Message of the calling thread's last failed call ("" if none). */
const char *swg_last_error(void);
/* Library version string. */
const char *swg_version(void);
/* Number of kernels this library launched since load (all entry points). */
long long swg_kernel_launches(void);

/* ------------------------------------------------------------- mesh ------
 * MPAS mesh tables, as in struct MPASMesh (src/mesh/mpas_mesh.hpp:7-71).
 * Host pointers; only the fields the hot path reads are required.  maxedges
 * is 6 (mpas_mesh.hpp:8); edges_on_edge / weights_on_edge rows have 12
 * slots of which nedges_on_edge[e] are used.  edge_mask may be NULL (all
 * ones, which is what MPASMesh::finalize_mesh sets, mpas_mesh.cpp:50);
 * mesh_scaling_del2/4 may be NULL (all ones, mpas_mesh.cpp:48-49). */
typedef struct swg_mesh_desc {
  int ncells, nedges, nvertices, nlayers;
  const int *nedges_on_cell;      /* [C]      */
  const int *edges_on_cell;       /* [C][6]   */
  const int *nedges_on_edge;      /* [E]      */
  const int *edges_on_edge;       /* [E][12]  */
  const int *cells_on_edge;       /* [E][2]   */
  const int *vertices_on_edge;    /* [E][2]   */
  const int *edges_on_vertex;     /* [V][3]   */
  const int *cells_on_vertex;     /* [V][3]   */
  const double *area_cell;        /* [C]      */
  const double *edge_sign_on_cell;   /* [C][6] */
  const double *dc_edge, *dv_edge;   /* [E]    */
  const double *weights_on_edge;     /* [E][12] */
  const double *area_triangle;       /* [V]    */
  const double *kiteareas_on_vertex; /* [V][3] */
  const double *edge_sign_on_vertex; /* [V][3] */
  const double *mesh_scaling_del2;   /* [E] or NULL */
  const double *mesh_scaling_del4;   /* [E] or NULL */
  const double *edge_mask;           /* [E][K] or NULL */
  /* levels per column summed by the diagnostics
   * (shallow_water_diagnostics.cpp:23,52,76); NULL = nlayers everywhere */
  const int *max_level_cell;         /* [C] in [0, K] or NULL */
  const int *max_level_vertex_bot;   /* [V] in [0, K] or NULL */
} swg_mesh_desc;

/* Host tables of the doubly periodic planar hexagonal mesh, identical to
 * PlanarHexagonalMesh(nx, ny, dc, nlayers) (planar_hexagonal_mesh.cpp:8-398,
 * mpas_mesh.cpp:5-57).  Caller-allocated arrays, sizes C = nx*ny, E = 3C,
 * V = 2C; any pointer may be NULL to skip that table. */
typedef struct swg_hex_tables {
  int *nedges_on_cell, *edges_on_cell, *cells_on_cell, *vertices_on_cell;
  int *kite_index_on_cell;
  int *nedges_on_edge, *edges_on_edge, *cells_on_edge, *vertices_on_edge;
  int *edges_on_vertex, *cells_on_vertex;
  double *area_cell, *x_cell, *y_cell, *edge_sign_on_cell;
  double *dc_edge, *dv_edge, *angle_edge, *x_edge, *y_edge, *weights_on_edge;
  double *area_triangle, *x_vertex, *y_vertex, *kiteareas_on_vertex;
  double *edge_sign_on_vertex;
} swg_hex_tables;

/* replaces PlanarHexagonalMesh::PlanarHexagonalMesh + compute_mesh_arrays +
 * MPASMesh::finalize_mesh (planar_hexagonal_mesh.cpp:8-62,168-398;
 * mpas_mesh.cpp:5-57).  Host only, no GPU needed.  ny odd reproduces the
 * reference's serial construction order (the Kokkos version races there). */
int swg_planar_hex_mesh_build(int nx, int ny, double dc, swg_hex_tables *out,
                              double *period_x, double *period_y);

/* Uploads the tables and derives the K-independent coefficient tables the
 * kernels use.  replaces the device-resident MPASMesh views. */
int swg_mesh_create(const swg_mesh_desc *desc, swg_mesh *out);
int swg_mesh_destroy(swg_mesh mesh);

/* ------------------------------------------------------------ state ------
 * replaces ShallowWaterState (shallow_water_state.hpp:9-16,
 * shallow_water_state.cpp:7-14): h_cell [C][K], vn_edge [E][K],
 * tr_cell [T][C][K], device resident, zero-initialised. */
int swg_state_create(swg_mesh mesh, int ntracers, swg_state *out);
int swg_state_destroy(swg_state state);
/* host -> device; tr may be NULL when ntracers == 0 */
int swg_state_upload(swg_state state, const double *h, const double *vn,
                     const double *tr, void *stream);
/* device -> host, synchronous */
int swg_state_download(swg_state state, double *h, double *vn, double *tr,
                       void *stream);
/* device pointers of the three arrays (any out-pointer may be NULL) */
int swg_state_device_ptrs(swg_state state, double **h, double **vn,
                          double **tr);
/* dst <- src, device to device (deep_copy of the three views) */
int swg_state_copy(swg_state dst, swg_state src, void *stream);
int swg_state_fill(swg_state state, double value, void *stream);

/* ------------------------------------------------------------ model ------
 * replaces ShallowWaterParams (shallow_water_params.hpp:7-18). */
typedef struct swg_params {
  double f0, grav, drag_coeff, visc_del2, visc_del4, eddy_diff2, eddy_diff4;
  int ntracers, disable_h_tendency, disable_vn_tendency;
} swg_params;

/* replaces ShallowWaterModel::ShallowWaterModel (shallow_water_model.cpp:5-41):
 * each dissipation term is enabled when its coefficient is > 0. */
int swg_model_create(swg_mesh mesh, const swg_params *params, swg_model *out);
int swg_model_destroy(swg_model model);

/* Model variants beside the reference's live model.  Both come from its
 * un-built hierarchical source (shallow_water_hierarchical.cpp):
 *   linear:     LinearShallowWaterModel (:676-775), the shallow-water
 *               equations linearised about a resting layer of thickness h0:
 *               h_t = -h0 div(vn), vn_t = f0 sum_j w_j vn_j - g grad h.
 *               Dissipation coefficients are ignored; ntracers must be 0.
 *   apply_drag: bottom drag -drag_coeff sqrt(ke_c0 + ke_c1) vn / mean_h on
 *               the lowest level of every edge (the term commented out at
 *               :479-486).  The reference's live model declares drag_coeff
 *               (shallow_water_params.hpp:10) but never applies it, which is
 *               what swg_model_create reproduces; the drag is opt-in. */
typedef struct swg_model_options {
  int linear;
  double h0;
  int apply_drag;
} swg_model_options;
/* swg_model_create with options (NULL = swg_model_create).  Linear models and
 * models with drag are not differentiated (swg_adjoint_create rejects them);
 * linear models are not batched. */
int swg_model_create_ex(swg_mesh mesh, const swg_params *params,
                        const swg_model_options *opts, swg_model *out);
/* replaces LinearShallowWaterModel::LinearShallowWaterModel(mesh, params)
 * (shallow_water_hierarchical.cpp:676-678; h0 = LinearShallowWaterParams::
 * m_h0) */
int swg_linear_model_create(swg_mesh mesh, const swg_params *params, double h0,
                            swg_model *out);

/* The model's tendency terms, in the order of the reference's members
 * (shallow_water_model.hpp:19-29). */
#define SWG_TERM_THICKNESS_HADV 0   /* ThicknessHorzAdvOnCell          */
#define SWG_TERM_PV_FLUX 1          /* PotentialVortFluxOnEdge         */
#define SWG_TERM_KE_GRAD 2          /* KineticEnergyGradOnEdge         */
#define SWG_TERM_SSH_GRAD 3         /* SSHGradOnEdge                   */
#define SWG_TERM_VEL_DIFF 4         /* VelocityDiffusionOnEdge         */
#define SWG_TERM_VEL_HYPERDIFF 5    /* VelocityHyperDiffusionOnEdge    */
#define SWG_TERM_TRACER_HADV 6      /* TracerHorzAdvOnCell             */
#define SWG_TERM_TRACER_DIFF 7      /* TracerDiffusionOnCell           */
#define SWG_TERM_TRACER_HYPERDIFF 8 /* TracerHyperDiffusionOnCell      */
#define SWG_NTERMS 9
/* replaces setting / reading a term member's m_enabled (read at compute
 * time by shallow_water_model.cpp:43-311: replace zeroes the tendency, then
 * each enabled term adds to it).  Switching a term off always works;
 * switching on a dissipation term whose coefficient was 0 at create time is
 * SWG_ERR_ARG (it adds nothing and its intermediates were not allocated).
 * A switch applies to later evaluations and steps (steppers recapture their
 * graph); batches and adjoints copy the terms when created, and the
 * adjoint refuses a model whose terms differ from create's. */
int swg_model_set_term_enabled(swg_model model, int term, int enabled);
int swg_model_term_enabled(swg_model model, int term, int *enabled);

/* replaces the virtual ShallowWaterModel::additional_tendency hook
 * (shallow_water_model.hpp:42-44).  Called on the host after the built-in
 * terms of every tendency evaluation with device pointers and the stream the
 * evaluation runs on; it adds its forcing with its own kernels. */
typedef void (*swg_forcing_fn)(void *user, double *h_tend, double *vn_tend,
                               const double *h, const double *vn, double t,
                               void *stream);
int swg_model_set_forcing(swg_model model, swg_forcing_fn fn, void *user);

/* replaces ShallowWaterModel::compute_tendency(tend, state, t, add_mode)
 * (shallow_water_model.cpp:313-347). */
int swg_compute_tendency(swg_model model, swg_state tend, swg_state state,
                         double t, int add_mode, void *stream);

/* The model's auxiliary state and per-field tendencies, as the reference
 * splits compute_tendency (shallow_water_model.cpp:313-347).
 * swg_model_compute_aux replaces m_aux_state.compute(h, vn, tr, f_vertex,
 * mesh) (shallow_water_auxstate.cpp:12-50): device arrays of the model's
 * layout.  Every tendency evaluation and step also leaves its last
 * auxiliary state in the model.  The per-field calls replace
 * compute_h_tendency / compute_vn_tendency / compute_tr_tendency
 * (shallow_water_model.hpp:36-41, shallow_water_model.cpp:43-311): each reads
 * the intermediates of the last auxiliary computation (mean thickness,
 * vorticities, kinetic energy, divergence, normalised tracers) and the
 * normal velocity vn it is given (and the velocity tendency also its h, for
 * the SSH gradient), honours the term switches and add_mode (REPLACE zeroes
 * the field first), and runs no additional_tendency hook.  As in the
 * reference, the tracer call is not given h and does not read tr: the
 * normalised tracers come from the auxiliary state.  The velocity tendency
 * needs a model created with the velocity tendency enabled (SWG_ERR_STATE
 * otherwise).  The linear model (swg_linear_model_create) keeps no
 * auxiliary state: its h and vn calls read h and vn directly. */
int swg_model_compute_aux(swg_model model, const double *h, const double *vn,
                          const double *tr, void *stream);
int swg_compute_h_tendency(swg_model model, double *h_tend, const double *h,
                           const double *vn, int add_mode, void *stream);
int swg_compute_vn_tendency(swg_model model, double *vn_tend, const double *h,
                            const double *vn, int add_mode, void *stream);
int swg_compute_tr_tendency(swg_model model, double *tr_tend, const double *tr,
                            const double *vn, int add_mode, void *stream);

/* No counterpart in the reference.  For callers that cannot allocate device
 * memory while they run (a host framework that owns the whole device pool,
 * or code that must avoid the synchronisation an allocation brings): the
 * same tendency as swg_compute_tendency (REPLACE or INCREMENT into the
 * caller's arrays, no additional_tendency hook), with the parameter tables
 * and all intermediate fields kept in one static device array of
 * SWG_NOALLOC_SCRATCH_BYTES (64 MiB) compiled into the library instead of
 * model-owned buffers.  Inputs h [C][K], vn [E][K], tr [T][C][K] and outputs
 * h_tend, vn_tend, tr_tend are device pointers; tr/tr_tend may be NULL when
 * params->ntracers == 0.  It calls no cudaMalloc/cudaFree or other
 * allocating routine.  The array itself is device memory that CUDA commits
 * when it loads the library's device code into a context: under the default
 * lazy module loading (CUDA_MODULE_LOADING=LAZY) that happens inside the
 * first launch of one of this library's kernels in the context, which may be
 * this call.  A caller that reserves the whole pool should therefore make a
 * first call (or any other call of this library that launches a kernel) at
 * start-up, before it reserves the pool.  Meshes and parameter sets whose
 * scratch exceeds the maximum are rejected with SWG_ERR_ARG (64x64 cells x
 * 64 levels with one tracer and del2 viscosity fits).  The first call in
 * each CUDA context looks up the array's address with the device current
 * and caches it under the context's unique ID, so calls in another context
 * (non-primary, or re-created after cudaDeviceReset) look it up again; make
 * that first call before any stream capture.  Its launches are never timed
 * by swg_profile_enable (that would create events).  All calls share the
 * array: calls that overlap on the GPU (unordered streams) race on it. */
#define SWG_NOALLOC_SCRATCH_BYTES (64ull << 20)
int swg_compute_tendency_noalloc(swg_mesh mesh, const swg_params *params,
                                 const double *h, const double *vn,
                                 const double *tr, double *h_tend,
                                 double *vn_tend, double *tr_tend,
                                 int add_mode, void *stream);

/* Named auxiliary field of the last tendency evaluation, device pointer and
 * element count.  Names: "q_vertex" ((rvort+f)/h at vertices), "rvort_vertex",
 * "vel_div_cell", "ke_cell", "norm_tr_cell", "thick_flux_edge"
 * (mean h * vn), "mean_h_edge", "pv_edge" (sum of the two vertex q),
 * "vel_del2_edge", "vel_del2_rvort_vertex", "vel_del2_div_cell",
 * "tracer_del2_cell".  Fields a configuration does not need stay unwritten.
 * "f_vertex" [V] is the model's Coriolis parameter per vertex, the
 * reference's m_f_vertex (shallow_water_model.hpp:32, filled with f0 by
 * shallow_water_model.cpp:39): the caller may write it (through a cast, e.g.
 * a beta plane) and every later evaluation reads it; the linear model uses
 * f0 instead. */
int swg_model_aux(swg_model model, const char *name, const double **ptr,
                  long long *count);

/* ---------------------------------------------------------- steppers -----
 * replaces RK4Stepper / LSRKStepper (time_stepper.hpp:16-38, rk4.cpp,
 * lsrk.cpp).  kind SWG_STEPPER_RK4 (nstages ignored) or SWG_STEPPER_LSRK
 * with nstages 5 (Carpenter-Kennedy) or 1 (forward Euler). */
int swg_stepper_create(swg_model model, int kind, int nstages,
                       swg_stepper *out);
int swg_stepper_destroy(swg_stepper stepper);
/* nsteps calls of TimeStepper::do_step(t0 + s*dt, dt, state)
 * (time_stepper.hpp:10-11), in place on `state`.  use_graph != 0 replays a
 * CUDA graph of one step (ignored when a forcing hook is set). */
int swg_step(swg_stepper stepper, swg_state state, double t0, double dt,
             int nsteps, int use_graph, void *stream);

/* ---------------------------------------------- host-resident states -----
 * Steps a state that lives in host memory, for a host program that owns the
 * state between steps (no counterpart in the reference, whose Kokkos views
 * live in the execution space's memory).  The arrays have the layout of
 * swg_state_upload: h [C][K], vn [E][K], tr [T][C][K].
 * Every tendency term reads and writes one level at a time, so the levels
 * are cut into chunks of `level_chunk` levels (the last chunk takes the
 * rest; <= 0 or >= K: one chunk).  Each chunk is advanced by its own level
 * slice of the model.  The chunks are pipelined on three streams: chunk c+1
 * is copied in while chunk c is computed and chunk c-1 is copied out.
 * Copies overlap only from page-locked host memory (swg_host_alloc or
 * cudaHostAlloc); pageable arrays work but serialise.  When the arrays are
 * mapped into the device address space (swg_host_alloc, cudaHostAlloc
 * under unified addressing), the first chunk's copy-in and the last
 * chunk's copy-out, which no compute overlaps, run as SM copy kernels,
 * which move short level rows several times faster than the copy engines.
 * Results are bitwise equal to swg_state_upload + swg_step + swg_state_download
 * on the same model.  Each call reads the model's term switches and its
 * f_vertex.  The model must have no forcing hook, because the hook would see
 * level slices.  The model must outlive the stepper.  kind and nstages are
 * those of swg_stepper_create. */
int swg_host_stepper_create(swg_model model, int kind, int nstages,
                            int level_chunk, swg_host_stepper *out);
/* the same with chunk sizes given one by one (levels[0..nchunks), each >= 1,
 * adding up to K).  Smaller first and last chunks shorten the copy-in that
 * precedes the first compute and the copy-out that follows the last. */
int swg_host_stepper_create_levels(swg_model model, int kind, int nstages,
                                   int nchunks, const int *levels,
                                   swg_host_stepper *out);
int swg_host_stepper_destroy(swg_host_stepper hs);
/* levels per chunk of the stepper's chunks (n entries; *n = count if NULL) */
int swg_host_stepper_chunks(swg_host_stepper hs, int *levels, int *n);
/* nsteps steps of size dt from t0, in place on the host arrays.  Ordered
 * after the work already queued on `stream`; returns once the arrays hold
 * the result.  tr may be NULL when the model has no tracers. */
int swg_host_step(swg_host_stepper hs, double *h, double *vn, double *tr,
                  double t0, double dt, int nsteps, void *stream);
/* page-locked host memory (cudaHostAlloc) for the arrays above */
int swg_host_alloc(unsigned long long bytes, void **out);
int swg_host_free(void *p);

/* ----------------------------------------------------------- batches -----
 * Ensembles of independent members with uneven mesh size, level count and
 * tracer count, advanced together (no counterpart in the reference, which
 * runs one instance per process; each member's step is the reference's
 * do_step).  Members are (model, state) pairs whose models have no forcing
 * hook and share the edges-on-edge width; the batch owns the stepper scratch
 * of every member.  One RK stage of all members is one persistent
 * cooperative kernel (six passes separated by bounded grid barriers), or one
 * launch per pass, whichever launch configuration is selected. */
/* The batch keeps the member handles (and a CUDA graph of their device
 * arrays): the models and states must outlive it, and no model or state may
 * appear in two members (SWG_ERR_ARG). */
int swg_batch_create(int nmembers, const swg_model *models,
                     const swg_state *states, int kind, int nstages,
                     swg_batch *out);
int swg_batch_destroy(swg_batch batch);
/* nsteps steps of every member (dt shared), asynchronous on `stream`;
 * use_graph != 0 replays a CUDA graph of one step. */
int swg_batch_step(swg_batch batch, double t0, double dt, int nsteps,
                   int use_graph, void *stream);
/* Synchronises `stream` and reports SWG_ERR_TIMEOUT if a grid-barrier wait
 * expired since the last check (the kernel then returned early). */
int swg_batch_check(swg_batch batch, void *stream);
/* Launch configurations: count, explicit choice, and autotuning (times
 * `reps` steps of every configuration on the batch itself and keeps the
 * fastest; the timed steps advance the members). */
int swg_batch_config_count(void);
int swg_batch_set_config(swg_batch batch, int config);
int swg_batch_autotune(swg_batch batch, double dt, int reps, void *stream,
                       int *best, double *best_ms_per_step);
/* Failure-detection test: launches a wait that nothing releases with a
 * limit of limit_ms (<= 2000) and returns the resulting SWG_ERR_TIMEOUT. */
int swg_batch_selftest_timeout(swg_batch batch, double limit_ms,
                               void *stream);

/* ------------------------------------------ adjoint and tangent-linear ----
 * Differentiation of the RK4 or low-storage RK step (no counterpart in the
 * reference).  An adjoint object is tied to a model (any MPAS tables, edge
 * mask, mesh scaling and dv < dc/4 included; not a model with a forcing
 * hook, the linear model or the drag) and owns `nsnapshots` state
 * checkpoints for the binomial checkpointing schedule, two step tapes and
 * the adjoint work arrays.  Tendency level, in the style of an autograd
 * Function's jvp/vjp:
 *   swg_tlm_tendency: dtend = J(x) dx        (exact forward-mode derivative)
 *   swg_adj_tendency: lambda = J(x)^T mu     (hand-written reverse mode)
 * Trajectory level (the adjoint's stepper, dt fixed):
 *   swg_tlm_apply:   dx <- d x_N (propagated tangent of nsteps steps)
 *   swg_adj_forward: runs nsteps steps from state0 storing checkpoints,
 *                    writes x_N to final_out;
 *   swg_adj_backward: lambda (in: dL/dx_N) <- dL/dx_0.
 * Every call differentiates the model's terms as they are switched
 * (swg_model_set_term_enabled) when it runs; swg_adj_backward refuses
 * (SWG_ERR_STATE) a term set that differs from the one its forward sweep
 * ran with. */
int swg_adjoint_create(swg_model model, int nsnapshots, swg_adjoint *out);
/* the same for another stepper: SWG_STEPPER_RK4 (nstages ignored) or
 * SWG_STEPPER_LSRK with nstages 5 or 1 (lsrk.cpp:16-33, 36-89) */
int swg_adjoint_create_stepper(swg_model model, int nsnapshots, int kind,
                               int nstages, swg_adjoint *out);
int swg_adjoint_destroy(swg_adjoint adj);
int swg_tlm_tendency(swg_adjoint adj, swg_state x, swg_state dx,
                     swg_state dtend_out, void *stream);
int swg_adj_tendency(swg_adjoint adj, swg_state x, swg_state mu,
                     swg_state lambda_out, void *stream);
int swg_tlm_apply(swg_adjoint adj, swg_state x0, swg_state dx, double t0,
                  double dt, int nsteps, void *stream);
/* nsteps <= 10000 (SWG_ERR_ARG above: the schedule planner's limit);
 * SWG_ERR_BUDGET when nsnapshots is so small that the schedule would re-run
 * more than 32 plain steps per step (swg_checkpoint_cost > 32 nsteps). */
int swg_adj_forward(swg_adjoint adj, swg_state state0, double t0, double dt,
                    int nsteps, swg_state final_out, void *stream);
int swg_adj_backward(swg_adjoint adj, swg_state lambda, void *stream);
/* Batched ensemble adjoints: members with uneven sizes, each with its own
 * adjoint object (so its own checkpoint budget and schedule), advanced
 * together: the schedules are interleaved one action at a time and member m
 * runs on streams[m] (NULL array: the legacy stream), so the GPU executes the
 * members concurrently.  Results equal per-member swg_adj_forward/backward. */
int swg_adj_batch_forward(int n, const swg_adjoint *adjs,
                          const swg_state *states0, double t0, double dt,
                          int nsteps, const swg_state *finals,
                          void *const *streams);
int swg_adj_batch_backward(int n, const swg_adjoint *adjs,
                           const swg_state *lambdas, void *const *streams);
/* Batched adjoint ensemble (no counterpart in the reference): the members'
 * adjoints (distinct adjoints and models; uneven sizes, each with its own
 * snapshot budget) advanced together, every action of the checkpoint
 * schedule one batched launch per pass over the members.  Members with the
 * same schedule (step count, snapshot budget, stepper) and the same kernel
 * switches (edges-on-edge width, tracer diffusion) form a group that runs
 * in lockstep: plain advances as a batch of the members' states, taped
 * steps as batched tendency passes into the members' tapes, and the adjoint
 * of a step as batched adjoint passes.  Groups run on streams of their own;
 * `stream` orders the ensemble after earlier work on it and later work
 * after it.  Results equal each member's swg_adj_forward / swg_adj_backward
 * bit for bit, and swg_adj_info / swg_adj_grad_visc of a member report its
 * part.  The ensemble keeps device tables of its members: create it once
 * and reuse it. */
int swg_adj_ensemble_create(int n, const swg_adjoint *adjs,
                            swg_adj_ensemble *out);
int swg_adj_ensemble_destroy(swg_adj_ensemble ens);
int swg_adj_ensemble_forward(swg_adj_ensemble ens, const swg_state *states0,
                             double t0, double dt, int nsteps,
                             const swg_state *finals, void *stream);
int swg_adj_ensemble_backward(swg_adj_ensemble ens, const swg_state *lambdas,
                              void *stream);
/* number of groups, and (if group_of is not NULL) each member's group */
int swg_adj_ensemble_groups(swg_adj_ensemble ens, int *ngroups,
                            int *group_of);
/* plain (re-)advanced and taped steps of the last forward/backward pair;
 * every step is taped once, either from a restored or re-advanced state or
 * as a taped advance (a step whose tape is kept while its result continues
 * the advance).  No counterpart in the reference. */
int swg_adj_info(swg_adjoint adj, long long *plain_steps,
                 long long *taped_steps);
/* the same, plus how many of the taped steps were taped advances */
int swg_adj_info_ex(swg_adjoint adj, long long *plain_steps,
                    long long *taped_steps, long long *taped_advances);
/* device bytes of one snapshot (a state), of one tape (the stage inputs,
 * accumulator and intermediates of one step; the adjoint holds two), and
 * of everything the adjoint holds besides its tables.  No counterpart in
 * the reference. */
int swg_adj_memory(swg_adjoint adj, long long *snapshot_bytes,
                   long long *tape_bytes, long long *total_bytes);
/* Gradient of the loss whose dL/dx_N was given to the last swg_adj_backward
 * with respect to the del2 viscosity, host arrays (either may be NULL):
 * per edge, d L / d(visc_del2 * mesh_scaling_del2[e]); per cell, for a
 * per-cell field mapped to edges as visc_e = (visc_c0 + visc_c1) / 2
 * (realised through mesh_scaling_del2, vel_diff_edge.hpp:83-84).  Only the
 * momentum term is differentiated: with eddy_diff2 > 0 the same scaling
 * also enters tracer diffusion, which this gradient leaves out.
 * SWG_ERR_STATE until a backward sweep has completed. */
int swg_adj_grad_visc(swg_adjoint adj, double *grad_edge, double *grad_cell,
                      void *stream);
/* plain advances of the classic optimal binomial schedule with one tape
 * (Griewank-Walther; host only; -1 for nsteps outside [1, 10000] or
 * nsnapshots < 1).  The adjoint's own planner, which also tapes the last
 * step of a re-advance, needs fewer: swg_adj_plan. */
long long swg_checkpoint_cost(int nsteps, int nsnapshots);
/* the schedule the adjoint runs for nsteps steps, nsnapshots snapshots and
 * a stepper of nstages stages (4: RK4; 5 or 1: LSRK): plain advances and
 * taped advances, as swg_adj_info_ex reports them after a forward/backward
 * pair (host only).  No counterpart in the reference. */
int swg_adj_plan(int nsteps, int nsnapshots, int nstages,
                 long long *plain_steps, long long *taped_advances);
/* the same schedule as a list of actions (host only): *count actions, the
 * first max_actions of them written as (type, a, b) triples.  Types:
 * 0 advance `cur` from step a by b plain steps, 1 store `cur` in snapshot
 * a, 2 restore `cur` from snapshot a, 3 tape step a from `cur` into tape b
 * and reverse it, 4 taped advance of step a into tape b (its result
 * replaces `cur`), 5 reverse step a from tape b, 6 end of the forward sweep
 * (x_N in `cur`). */
int swg_adj_schedule(int nsteps, int nsnapshots, int nstages,
                     int max_actions, int *actions, int *count);

/* ----------------------------------------------------- measurement -----
 * FP64 issue rate of the current GPU (no counterpart in the reference): op
 * 0 DFMA, 1 DADD, 2 DMUL; every SM filled with resident threads, each
 * running 4 independent chains for `iters` iterations, timed with CUDA
 * events on `stream` (blocking).  *inst_per_s gets thread-instructions per
 * second, *ms (may be NULL) the timed kernel's duration.  The solver's
 * kernels are bound by this rate, not by HBM bandwidth. */
int swg_fp64_issue_rate(int op, int iters, double *inst_per_s, double *ms,
                        void *stream);

/* ------------------------------------------------------- diagnostics -----
 * replaces energy_integral / mass_integral / circulation_integral
 * (shallow_water_diagnostics.cpp:5-89).  Synchronous on `stream`. */
int swg_diag_mass(swg_model model, swg_state state, double *out, void *stream);
int swg_diag_energy(swg_model model, swg_state state, double *out,
                    void *stream);
int swg_diag_circulation(swg_model model, swg_state state, double *out,
                         void *stream);

/* ---------------------------------------------------------- profiling ----
 * Diagnostic (no reference counterpart): while enabled, every tendency
 * kernel is bracketed by a CUDA event pair on its stream and graph replay is
 * bypassed.  swg_profile_read synchronises those events and returns, per
 * kernel name (names: max_kernels x 32 chars), the summed milliseconds and
 * launch count, then clears the record. */
int swg_profile_enable(int on);
int swg_profile_read(int max_kernels, char *names, double *total_ms,
                     long long *launches, int *count);

/* Blocks until `stream` is idle; reports any pending CUDA error. */
int swg_sync(void *stream);

#ifdef __cplusplus
}
#endif
#endif
