/*
 * CPU oracle for the omega_playground shallow-water hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the
 * reference's algorithm, used as the checker by tests/, by the smoke() entry
 * point and as the timed CPU baseline ("port") in bench.py.  The product
 * (omega_playground_gb300) never links, loads or calls it.
 *
 * Every function follows the reference's expression order term by term
 * (default build: no OMEGA_KOKKOS_SIMD, inner-if kernels, vector_length 1)
 * and is compiled with -ffp-contract=off, so it is bit-identical to the
 * reference sources compiled with GCC in ISO C++17 mode.  Layout: FP64
 * [entity][k] row-major, tracers [l][cell][k], int32 connectivity.
 */
#ifndef SWE_ORACLE_H
#define SWE_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Mesh tables, mirroring MPASMesh (src/mesh/mpas_mesh.hpp:7-71).  All
 * pointers are caller-owned and must stay valid while a model uses them. */
typedef struct or_mesh {
  int nx, ny, ncells, nedges, nvertices, nlayers;
  double dc, period_x, period_y;
  int *nedges_on_cell;     /* [C]     */
  int *edges_on_cell;      /* [C][6]  */
  int *cells_on_cell;      /* [C][6]  */
  int *vertices_on_cell;   /* [C][6]  */
  int *kite_index_on_cell; /* [C][6]  */
  int *nedges_on_edge;     /* [E]     */
  int *edges_on_edge;      /* [E][12] */
  int *cells_on_edge;      /* [E][2]  */
  int *vertices_on_edge;   /* [E][2]  */
  int *edges_on_vertex;    /* [V][3]  */
  int *cells_on_vertex;    /* [V][3]  */
  double *area_cell, *x_cell, *y_cell;
  double *edge_sign_on_cell; /* [C][6] */
  double *dc_edge, *dv_edge, *angle_edge, *x_edge, *y_edge;
  double *weights_on_edge; /* [E][12] */
  double *mesh_scaling_del2, *mesh_scaling_del4; /* [E] */
  double *edge_mask;                             /* [E][K] */
  double *area_triangle, *x_vertex, *y_vertex;
  double *kiteareas_on_vertex; /* [V][3] */
  double *edge_sign_on_vertex; /* [V][3] */
  /* levels per column summed by the diagnostics; NULL = nlayers */
  int *max_level_cell;         /* [C] */
  int *max_level_vertex_bot;   /* [V] */
} or_mesh;

/* ShallowWaterParams (src/model/shallow_water_params.hpp:7-18). */
typedef struct or_params {
  double f0, grav, drag_coeff, visc_del2, visc_del4, eddy_diff2, eddy_diff4;
  int ntracers, disable_h_tendency, disable_vn_tendency;
} or_params;

typedef struct or_model or_model;

/* Sizes of the doubly periodic planar hexagonal mesh. */
void or_planar_hex_sizes(int nx, int ny, int *ncells, int *nedges,
                         int *nvertices);
/* Fills every table of `m` (arrays preallocated by the caller with the sizes
 * above; edge_mask holds nedges*nlayers values). */
void or_planar_hex_build(or_mesh *m, int nx, int ny, double dc, int nlayers);

or_model *or_model_create(const or_mesh *m, const or_params *p);
/* linear != 0: LinearShallowWaterModel with resting thickness h0
 * (shallow_water_hierarchical.cpp:676-775; no tracers, no dissipation).
 * apply_drag != 0: the nonlinear model plus the bottom drag that
 * shallow_water_hierarchical.cpp:479-486 leaves commented out. */
or_model *or_model_create_ex(const or_mesh *m, const or_params *p, int linear,
                             double h0, int apply_drag);
void or_model_destroy(or_model *md);
/* Pointer to a named auxiliary array of the model (NULL if unknown); *n gets
 * its element count.  Names follow the reference's member names. */
double *or_model_aux(or_model *md, const char *name, size_t *n);

/* Sets the m_enabled of term `term` (0 ThicknessHorzAdvOnCell, 1 PV flux,
 * 2 KE gradient, 3 SSH gradient, 4 velocity del2, 5 velocity del4, 6 tracer
 * advection, 7 tracer del2, 8 tracer del4: shallow_water_model.hpp:19-29).
 * Returns 0, or 1 for an unknown term. */
int or_model_set_term(or_model *md, int term, int enabled);

/* ShallowWaterModel::compute_tendency (shallow_water_model.cpp:313-347).
 * add_mode: 0 replace, 1 increment. */
void or_compute_tendency(or_model *md, double *h_tend, double *vn_tend,
                         double *tr_tend, const double *h, const double *vn,
                         const double *tr, double t, int add_mode);

/* The split compute_tendency of the reference: the auxiliary state
 * (ShallowWaterAuxiliaryState::compute, shallow_water_auxstate.cpp:12-50)
 * and the per-field tendencies from it (compute_h_tendency,
 * compute_vn_tendency, compute_tr_tendency: shallow_water_model.cpp:43-311),
 * which read the aux state of the last or_aux_compute / or_compute_tendency
 * and their own arguments.  Nonlinear model only. */
void or_aux_compute(or_model *md, const double *h, const double *vn,
                    const double *tr);
void or_h_tendency(or_model *md, double *h_tend, const double *vn,
                   int add_mode);
void or_vn_tendency(or_model *md, double *vn_tend, const double *h,
                    const double *vn, int add_mode);
void or_tr_tendency(or_model *md, double *tr_tend, const double *vn,
                    int add_mode);

/* nsteps steps of RK4Stepper (kind 0) or LSRKStepper (kind 1, nstages 5 or
 * 1) starting at t0, in place on (h, vn, tr).  Stepper scratch persists in
 * the model across calls, like the reference's stepper members. */
int or_step(or_model *md, int kind, int nstages, double *h, double *vn,
            double *tr, double t0, double dt, int nsteps);

/* shallow_water_diagnostics.cpp:5-89 */
double or_mass_integral(or_model *md, const double *h);
double or_energy_integral(or_model *md, const double *h, const double *vn);
double or_circulation_integral(or_model *md, const double *vn);

/* Number of OpenMP threads the oracle runs with. */
int or_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
