/*
 * CPU oracle for the omega_playground shallow-water hot path (see
 * swe_oracle.h).  TEST INFRASTRUCTURE ONLY: the checker for tests/, smoke()
 * and the CPU-baseline leg of bench.py; the product never uses it.
 *
 * Each function restates one reference routine; the citation is the file and
 * line range (paths relative to the omega_playground checkout) whose
 * arithmetic it reproduces in the same association order.  Entity loops are
 * OpenMP-parallel; every output element is computed by one thread, so the
 * results do not depend on the thread count.  Reductions (diagnostics) are
 * serial so their summation order is the reference's serial order.
 */
#include "swe_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXEDGES 6

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ---------------------------------------------------------------- mesh --- */

void or_planar_hex_sizes(int nx, int ny, int *ncells, int *nedges,
                         int *nvertices) {
  /* planar_hexagonal_mesh.cpp:13-15 */
  *ncells = nx * ny;
  *nedges = 3 * nx * ny;
  *nvertices = 2 * nx * ny;
}

static int hex_cellidx(const or_mesh *m, int icol, int irow) {
  return irow * m->nx + icol; /* planar_hexagonal_mesh.cpp:64-67 */
}

/* planar_hexagonal_mesh.cpp:69-117: neighbour nb (0..5, counter-clockwise
 * from west) of cell (icol, irow); odd rows are shifted half a cell east. */
static int hex_cell_on_cell(const or_mesh *m, int icol, int irow, int nb) {
  int mx = icol == 0 ? m->nx - 1 : icol - 1;
  int px = icol == (m->nx - 1) ? 0 : icol + 1;
  int my = irow == 0 ? m->ny - 1 : irow - 1;
  int py = irow == (m->ny - 1) ? 0 : irow + 1;
  static const int even_dx[6] = {-1, -1, 0, 1, 0, -1};
  static const int odd_dx[6] = {-1, 0, 1, 1, 1, 0};
  static const int dy[6] = {0, -1, -1, 0, 1, 1};
  int dx = (irow % 2 == 0) ? even_dx[nb] : odd_dx[nb];
  int c = dx < 0 ? mx : (dx > 0 ? px : icol);
  int r = dy[nb] < 0 ? my : (dy[nb] > 0 ? py : irow);
  return hex_cellidx(m, c, r);
}

/* planar_hexagonal_mesh.cpp:119-141 */
static int hex_edge_on_cell(const or_mesh *m, int icell, int icol, int irow,
                            int nb) {
  if (nb < 3)
    return 3 * icell + nb;
  return 3 * hex_cell_on_cell(m, icol, irow, nb) + (nb - 3);
}

/* planar_hexagonal_mesh.cpp:143-166 */
static int hex_vertex_on_cell(const or_mesh *m, int icell, int icol, int irow,
                              int nb) {
  switch (nb) {
  case 0: return 2 * icell;
  case 1: return 2 * icell + 1;
  case 2: return 2 * hex_cell_on_cell(m, icol, irow, 2);
  case 3: return 2 * hex_cell_on_cell(m, icol, irow, 3) + 1;
  case 4: return 2 * hex_cell_on_cell(m, icol, irow, 3);
  default: return 2 * hex_cell_on_cell(m, icol, irow, 4) + 1;
  }
}

void or_planar_hex_build(or_mesh *m, int nx, int ny, double dc, int nlayers) {
  /* constructor: planar_hexagonal_mesh.cpp:8-17 (vector_length 1: no level
   * padding) */
  m->nx = nx;
  m->ny = ny;
  m->dc = dc;
  m->nlayers = nlayers;
  or_planar_hex_sizes(nx, ny, &m->ncells, &m->nedges, &m->nvertices);
  m->period_x = nx * dc;
  m->period_y = ny * dc * sqrt(3.0) / 2;
  const int C = m->ncells, E = m->nedges, V = m->nvertices;
  /* Kokkos views are zero-initialised; the two unused edges_on_edge and
   * weights_on_edge slots (10, 11) stay 0. */
  memset(m->edges_on_edge, 0, sizeof(int) * (size_t)E * 12);
  memset(m->weights_on_edge, 0, sizeof(double) * (size_t)E * 12);
  memset(m->cells_on_edge, 0, sizeof(int) * (size_t)E * 2);
  memset(m->vertices_on_edge, 0, sizeof(int) * (size_t)E * 2);
  memset(m->cells_on_vertex, 0, sizeof(int) * (size_t)V * 3);
  memset(m->edges_on_vertex, 0, sizeof(int) * (size_t)V * 3);
  memset(m->kite_index_on_cell, 0, sizeof(int) * (size_t)C * 6);

  /* compute_mesh_arrays: planar_hexagonal_mesh.cpp:169-321.  Serial in the
   * reference's MDRange order (irow outer, icol inner), so for odd ny the
   * doubly written slots keep the serial last writer. */
  for (int irow = 0; irow < ny; ++irow) {
    for (int icol = 0; icol < nx; ++icol) {
      const int c = hex_cellidx(m, icol, irow);
      int *eoc = m->edges_on_cell + 6 * c;
      int *voc = m->vertices_on_cell + 6 * c;
      m->nedges_on_cell[c] = 6;
      for (int j = 0; j < MAXEDGES; ++j) {
        m->cells_on_cell[6 * c + j] = hex_cell_on_cell(m, icol, irow, j);
        eoc[j] = hex_edge_on_cell(m, c, icol, irow, j);
        voc[j] = hex_vertex_on_cell(m, c, icol, irow, j);
      }
      for (int j = 0; j < 3; ++j)
        m->cells_on_edge[2 * eoc[j] + 1] = c;
      for (int j = 3; j < MAXEDGES; ++j)
        m->cells_on_edge[2 * eoc[j] + 0] = c;
      /* :187-198 */
      m->vertices_on_edge[2 * eoc[0] + 0] = voc[1];
      m->vertices_on_edge[2 * eoc[0] + 1] = voc[0];
      m->vertices_on_edge[2 * eoc[1] + 0] = voc[2];
      m->vertices_on_edge[2 * eoc[1] + 1] = voc[1];
      m->vertices_on_edge[2 * eoc[2] + 0] = voc[3];
      m->vertices_on_edge[2 * eoc[2] + 1] = voc[2];
      /* :200-264: slots 0-4 of edges 3,4,5 and slots 5-9 of edges 0,1,2
       * list the cell's other five edges counter-clockwise. */
      for (int i = 3; i < 6; ++i)
        for (int s = 0; s < 5; ++s)
          m->edges_on_edge[12 * eoc[i] + s] = eoc[(i + 1 + s) % 6];
      for (int i = 0; i < 3; ++i)
        for (int s = 0; s < 5; ++s)
          m->edges_on_edge[12 * eoc[i] + 5 + s] = eoc[(i + 1 + s) % 6];
      /* :266-300 (before the 1/sqrt(3) scaling) */
      static const double w3[5] = {1. / 3, 1. / 6, 0, 1. / 6, 1. / 3};
      static const double w4[5] = {1. / 3, -1. / 6, 0, 1. / 6, -1. / 3};
      static const double w5[5] = {-1. / 3, -1. / 6, 0, -1. / 6, -1. / 3};
      for (int s = 0; s < 5; ++s) {
        m->weights_on_edge[12 * eoc[3] + s] = w3[s];
        m->weights_on_edge[12 * eoc[4] + s] = w4[s];
        m->weights_on_edge[12 * eoc[5] + s] = w5[s];
        m->weights_on_edge[12 * eoc[0] + 5 + s] = w3[s];
        m->weights_on_edge[12 * eoc[1] + 5 + s] = w4[s];
        m->weights_on_edge[12 * eoc[2] + 5 + s] = w5[s];
      }
      /* :302-320 */
      m->cells_on_vertex[3 * voc[1] + 2] = c;
      m->cells_on_vertex[3 * voc[3] + 0] = c;
      m->cells_on_vertex[3 * voc[5] + 1] = c;
      m->cells_on_vertex[3 * voc[0] + 0] = c;
      m->cells_on_vertex[3 * voc[2] + 1] = c;
      m->cells_on_vertex[3 * voc[4] + 2] = c;
      m->edges_on_vertex[3 * voc[0] + 0] = eoc[0];
      m->edges_on_vertex[3 * voc[1] + 0] = eoc[0];
      m->edges_on_vertex[3 * voc[2] + 2] = eoc[1];
      m->edges_on_vertex[3 * voc[1] + 2] = eoc[1];
      m->edges_on_vertex[3 * voc[2] + 1] = eoc[2];
      m->edges_on_vertex[3 * voc[3] + 1] = eoc[2];
    }
  }
  /* scale_weights: :323-327 */
  for (int e = 0; e < E; ++e)
    for (int j = 0; j < 2 * MAXEDGES; ++j)
      m->weights_on_edge[12 * e + j] *= 1. / sqrt(3.0);

  /* M_PI (the reference's omega::pi), spelled out for strict ISO C */
  const double pi = 3.14159265358979323846;
  /* compute_cell_arrays: :329-376 */
  for (int irow = 0; irow < ny; ++irow) {
    for (int icol = 0; icol < nx; ++icol) {
      const int c = hex_cellidx(m, icol, irow);
      const int *eoc = m->edges_on_cell + 6 * c;
      const int *voc = m->vertices_on_cell + 6 * c;
      m->area_cell[c] = dc * dc * sqrt(3.0) / 2;
      if (irow % 2 == 0) {
        m->x_cell[c] = dc * icol + dc / 2;
        m->y_cell[c] = dc * (irow + 1) * sqrt(3.0) / 2;
      } else {
        m->x_cell[c] = dc * (icol + 1);
        m->y_cell[c] = dc * (irow + 1) * sqrt(3.0) / 2;
      }
      m->x_edge[eoc[0]] = m->x_cell[c] - dc / 2;
      m->y_edge[eoc[0]] = m->y_cell[c];
      m->x_edge[eoc[1]] = m->x_cell[c] - dc / 2 * cos(pi / 3);
      m->y_edge[eoc[1]] = m->y_cell[c] - dc / 2 * sin(pi / 3);
      m->x_edge[eoc[2]] = m->x_cell[c] + dc / 2 * cos(pi / 3);
      m->y_edge[eoc[2]] = m->y_cell[c] - dc / 2 * sin(pi / 3);
      m->angle_edge[eoc[0]] = 0;
      m->angle_edge[eoc[1]] = pi / 3;
      m->angle_edge[eoc[2]] = 2 * pi / 3;
      m->x_vertex[voc[0]] = m->x_cell[c] - dc / 2;
      m->y_vertex[voc[0]] = m->y_cell[c] + dc * sqrt(3.0) / 6;
      m->x_vertex[voc[1]] = m->x_cell[c] - dc / 2;
      m->y_vertex[voc[1]] = m->y_cell[c] - dc * sqrt(3.0) / 6;
    }
  }
  /* compute_edge_arrays: :378-385 */
  for (int e = 0; e < E; ++e) {
    m->nedges_on_edge[e] = 10;
    m->dc_edge[e] = dc;
    m->dv_edge[e] = m->dc_edge[e] * sqrt(3.0) / 3;
  }
  /* compute_vertex_arrays: :387-395 */
  for (int v = 0; v < V; ++v) {
    m->area_triangle[v] = dc * dc * sqrt(3.0) / 4;
    for (int j = 0; j < 3; ++j)
      m->kiteareas_on_vertex[3 * v + j] = dc * dc * sqrt(3.0) / 12;
  }
  /* finalize_mesh: mpas_mesh.cpp:5-57 */
  for (int c = 0; c < C; ++c) {
    for (int j = 0; j < m->nedges_on_cell[c]; ++j)
      m->edge_sign_on_cell[6 * c + j] =
          m->cells_on_edge[2 * m->edges_on_cell[6 * c + j]] == c ? 1 : -1;
    for (int j = 0; j < m->nedges_on_cell[c]; ++j) {
      int jv = m->vertices_on_cell[6 * c + j];
      for (int l = 0; l < 3; ++l)
        if (m->cells_on_vertex[3 * jv + l] == c)
          m->kite_index_on_cell[6 * c + j] = l;
    }
  }
  for (int v = 0; v < V; ++v)
    for (int j = 0; j < 3; ++j)
      m->edge_sign_on_vertex[3 * v + j] =
          m->vertices_on_edge[2 * m->edges_on_vertex[3 * v + j]] == v ? -1 : 1;
  for (int e = 0; e < E; ++e) {
    m->mesh_scaling_del2[e] = 1;
    m->mesh_scaling_del4[e] = 1;
  }
  for (size_t i = 0; i < (size_t)E * nlayers; ++i)
    m->edge_mask[i] = 1;
}

/* --------------------------------------------------------------- model --- */

struct or_model {
  or_mesh m;
  or_params p;
  int en_vel_diff, en_vel_hyperdiff, en_tr_diff, en_tr_hyperdiff;
  /* the always-on terms' m_enabled (shallow_water_model.cpp:17-21,29) */
  int en_hadv, en_pv, en_ke, en_ssh, en_tr_hadv;
  /* variants from shallow_water_hierarchical.cpp: LinearShallowWaterModel
   * (h0) and the bottom drag that its nonlinear model leaves commented out */
  int linear, apply_drag;
  double h0;
  double *f_vertex;
  /* auxiliary state (shallow_water_auxstate.hpp:9-21) */
  double *rvort_vertex, *norm_rvort_vertex, *norm_pvort_vertex;
  double *norm_rvort_edge, *norm_pvort_edge, *mean_h_edge, *flux_h_edge;
  double *ke_cell, *vel_div_cell, *norm_tr_cell;
  /* term scratch (vel_hyperdiff_edge.hpp:109-111, tracer_hyperdiff_cell.hpp:11) */
  double *vel_del2_edge, *vel_del2_rvort_vertex, *vel_del2_div_cell;
  double *tracer_del2_cell;
  /* stepper scratch: LSRK m_tend; RK4 m_tend, m_provis_state, m_old_state */
  double *st_tend, *st_provis, *st_old;
  int st_kind, st_nstages;
};

static double *zalloc(size_t n) { return (double *)calloc(n ? n : 1, 8); }

or_model *or_model_create(const or_mesh *m, const or_params *p) {
  return or_model_create_ex(m, p, 0, 0.0, 0);
}

or_model *or_model_create_ex(const or_mesh *m, const or_params *p, int linear,
                             double h0, int apply_drag) {
  or_model *md = (or_model *)calloc(1, sizeof(or_model));
  md->m = *m;
  md->p = *p;
  md->linear = linear;
  md->h0 = h0;
  md->apply_drag = apply_drag && !linear;
  /* shallow_water_model.cpp:17-35 */
  md->en_vel_diff = p->visc_del2 > 0;
  md->en_vel_hyperdiff = p->visc_del4 > 0;
  md->en_tr_diff = p->eddy_diff2 > 0;
  md->en_tr_hyperdiff = p->eddy_diff4 > 0;
  md->en_hadv = md->en_pv = md->en_ke = md->en_ssh = md->en_tr_hadv = 1;
  const size_t K = m->nlayers, C = m->ncells, E = m->nedges, V = m->nvertices;
  const size_t T = p->ntracers;
  md->f_vertex = zalloc(V);
  for (size_t v = 0; v < V; ++v)
    md->f_vertex[v] = p->f0; /* :39 */
  md->rvort_vertex = zalloc(V * K);
  md->norm_rvort_vertex = zalloc(V * K);
  md->norm_pvort_vertex = zalloc(V * K);
  md->norm_rvort_edge = zalloc(E * K);
  md->norm_pvort_edge = zalloc(E * K);
  md->mean_h_edge = zalloc(E * K);
  md->flux_h_edge = zalloc(E * K);
  md->ke_cell = zalloc(C * K);
  md->vel_div_cell = zalloc(C * K);
  md->norm_tr_cell = zalloc(T * C * K);
  md->vel_del2_edge = zalloc(E * K);
  md->vel_del2_rvort_vertex = zalloc(V * K);
  md->vel_del2_div_cell = zalloc(C * K);
  md->tracer_del2_cell = zalloc(T * C * K);
  md->st_kind = -1;
  return md;
}

void or_model_destroy(or_model *md) {
  if (!md)
    return;
  double *ptrs[] = {md->f_vertex, md->rvort_vertex, md->norm_rvort_vertex,
                    md->norm_pvort_vertex, md->norm_rvort_edge,
                    md->norm_pvort_edge, md->mean_h_edge, md->flux_h_edge,
                    md->ke_cell, md->vel_div_cell, md->norm_tr_cell,
                    md->vel_del2_edge, md->vel_del2_rvort_vertex,
                    md->vel_del2_div_cell, md->tracer_del2_cell, md->st_tend,
                    md->st_provis, md->st_old};
  for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i)
    free(ptrs[i]);
  free(md);
}

double *or_model_aux(or_model *md, const char *name, size_t *n) {
  const size_t K = md->m.nlayers, C = md->m.ncells, E = md->m.nedges,
               V = md->m.nvertices, T = md->p.ntracers;
  struct {
    const char *name;
    double *ptr;
    size_t n;
  } tab[] = {
      {"rvort_vertex", md->rvort_vertex, V * K},
      {"norm_rvort_vertex", md->norm_rvort_vertex, V * K},
      {"norm_pvort_vertex", md->norm_pvort_vertex, V * K},
      {"norm_rvort_edge", md->norm_rvort_edge, E * K},
      {"norm_pvort_edge", md->norm_pvort_edge, E * K},
      {"mean_h_edge", md->mean_h_edge, E * K},
      {"flux_h_edge", md->flux_h_edge, E * K},
      {"ke_cell", md->ke_cell, C * K},
      {"vel_div_cell", md->vel_div_cell, C * K},
      {"norm_tr_cell", md->norm_tr_cell, T * C * K},
      {"vel_del2_edge", md->vel_del2_edge, E * K},
      {"vel_del2_rvort_vertex", md->vel_del2_rvort_vertex, V * K},
      {"vel_del2_div_cell", md->vel_del2_div_cell, C * K},
      {"tracer_del2_cell", md->tracer_del2_cell, T * C * K},
      {"f_vertex", md->f_vertex, V},
  };
  for (size_t i = 0; i < sizeof(tab) / sizeof(tab[0]); ++i)
    if (strcmp(tab[i].name, name) == 0) {
      *n = tab[i].n;
      return tab[i].ptr;
    }
  *n = 0;
  return NULL;
}

/* ShallowWaterAuxiliaryState::compute (shallow_water_auxstate.cpp:12-50). */
void or_aux_compute(or_model *md, const double *h, const double *vn,
                    const double *tr) {
  const or_mesh *m = &md->m;
  const int K = m->nlayers, C = m->ncells, E = m->nedges, V = m->nvertices;
  const int T = md->p.ntracers;

  /* VorticityAuxVars::compute_vort_vertex (vorticity_aux.hpp:294-325) */
#pragma omp parallel for schedule(static)
  for (int v = 0; v < V; ++v) {
    const double inv_area_triangle = 1. / m->area_triangle[v];
    for (int k = 0; k < K; ++k) {
      double rvort = 0, thick = 0;
      for (int j = 0; j < 3; ++j) {
        const int je = m->edges_on_vertex[3 * v + j];
        const int jc = m->cells_on_vertex[3 * v + j];
        rvort += m->dc_edge[je] * inv_area_triangle *
                 m->edge_sign_on_vertex[3 * v + j] * vn[(size_t)je * K + k];
        thick += m->kiteareas_on_vertex[3 * v + j] * inv_area_triangle *
                 h[(size_t)jc * K + k];
      }
      const double inv_thick = 1. / thick;
      md->rvort_vertex[(size_t)v * K + k] = rvort;
      md->norm_rvort_vertex[(size_t)v * K + k] = inv_thick * rvort;
      md->norm_pvort_vertex[(size_t)v * K + k] = inv_thick * md->f_vertex[v];
    }
  }

  /* KineticAuxVars::compute_kinetic_cell (kinetic_aux.hpp:50-79) and
   * TracerAuxVars::compute_norm_tracer_cell (tracer_aux.hpp:181-201) */
#pragma omp parallel for schedule(static)
  for (int c = 0; c < C; ++c) {
    const double inv_area_cell = 1. / m->area_cell[c];
    for (int k = 0; k < K; ++k) {
      double ke = 0, div = 0;
      for (int j = 0; j < m->nedges_on_cell[c]; ++j) {
        const int je = m->edges_on_cell[6 * c + j];
        const double area_edge = m->dv_edge[je] * m->dc_edge[je];
        const double u = vn[(size_t)je * K + k];
        ke += inv_area_cell * area_edge * u * u * 0.25;
        div += inv_area_cell * m->dv_edge[je] * m->edge_sign_on_cell[6 * c + j] *
               u;
      }
      md->vel_div_cell[(size_t)c * K + k] = div;
      md->ke_cell[(size_t)c * K + k] = ke;
      for (int l = 0; l < T; ++l) {
        const double inv_h = 1. / h[(size_t)c * K + k];
        const size_t i = ((size_t)l * C + c) * K + k;
        md->norm_tr_cell[i] = tr[i] * inv_h;
      }
    }
  }

  /* ThicknessAuxVars::compute_thickness_edge (thickness_aux.hpp:123-142) and
   * VorticityAuxVars::compute_vort_edge (vorticity_aux.hpp:327-341) */
#pragma omp parallel for schedule(static)
  for (int e = 0; e < E; ++e) {
    const int c0 = m->cells_on_edge[2 * e], c1 = m->cells_on_edge[2 * e + 1];
    const int v0 = m->vertices_on_edge[2 * e], v1 = m->vertices_on_edge[2 * e + 1];
    for (int k = 0; k < K; ++k) {
      const size_t i = (size_t)e * K + k;
      const double mean = 0.5 * (h[(size_t)c0 * K + k] + h[(size_t)c1 * K + k]);
      md->mean_h_edge[i] = mean;
      md->flux_h_edge[i] = mean;
      md->norm_rvort_edge[i] = 0.5 * (md->norm_rvort_vertex[(size_t)v0 * K + k] +
                                      md->norm_rvort_vertex[(size_t)v1 * K + k]);
      md->norm_pvort_edge[i] = 0.5 * (md->norm_pvort_vertex[(size_t)v0 * K + k] +
                                      md->norm_pvort_vertex[(size_t)v1 * K + k]);
    }
  }
}

/* ShallowWaterModel::compute_h_tendency (shallow_water_model.cpp:71-84,
 * default inner-if kernel) with ThicknessHorzAdvOnCell
 * (thickness_hadv_cell.hpp:59-83); the flux thickness is m_flux_h_edge. */
void or_h_tendency(or_model *md, double *h_tend, const double *vn,
                   int add_mode) {
  const or_mesh *m = &md->m;
  const int K = m->nlayers, C = m->ncells;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < C; ++c) {
    const double inv_area_cell = 1. / m->area_cell[c];
    for (int k = 0; k < K; ++k) {
      const size_t i = (size_t)c * K + k;
      if (add_mode == 0)
        h_tend[i] = 0;
      if (!md->en_hadv) /* ThicknessHorzAdvOnCell switched off */
        continue;
      double accum = 0;
      for (int j = 0; j < m->nedges_on_cell[c]; ++j) {
        const int je = m->edges_on_cell[6 * c + j];
        accum -= m->dv_edge[je] * inv_area_cell *
                 m->edge_sign_on_cell[6 * c + j] *
                 md->flux_h_edge[(size_t)je * K + k] * vn[(size_t)je * K + k];
      }
      h_tend[i] += accum;
    }
  }
}

/* ShallowWaterModel::compute_vn_tendency (shallow_water_model.cpp:88-219). */
void or_vn_tendency(or_model *md, double *vn_tend, const double *h,
                    const double *vn, int add_mode) {
  const or_mesh *m = &md->m;
  const or_params *p = &md->p;
  const int K = m->nlayers, C = m->ncells, E = m->nedges, V = m->nvertices;

  if (md->en_vel_hyperdiff) {
    /* compute_vel_del2 (vel_hyperdiff_edge.hpp:237-261): 1/max(dv, dc/4) */
#pragma omp parallel for schedule(static)
    for (int e = 0; e < E; ++e) {
      const int c0 = m->cells_on_edge[2 * e], c1 = m->cells_on_edge[2 * e + 1];
      const int v0 = m->vertices_on_edge[2 * e],
                v1 = m->vertices_on_edge[2 * e + 1];
      const double dc_edge_inv = 1. / m->dc_edge[e];
      const double dvm = m->dv_edge[e] > 0.25 * m->dc_edge[e]
                             ? m->dv_edge[e]
                             : 0.25 * m->dc_edge[e];
      const double dv_edge_inv = 1. / dvm;
      for (int k = 0; k < K; ++k) {
        const double del2u =
            ((md->vel_div_cell[(size_t)c1 * K + k] -
              md->vel_div_cell[(size_t)c0 * K + k]) *
                 dc_edge_inv -
             (md->rvort_vertex[(size_t)v1 * K + k] -
              md->rvort_vertex[(size_t)v0 * K + k]) *
                 dv_edge_inv);
        md->vel_del2_edge[(size_t)e * K + k] = del2u;
      }
    }
    /* compute_vel_del2_rvort (vel_hyperdiff_edge.hpp:263-284) */
#pragma omp parallel for schedule(static)
    for (int v = 0; v < V; ++v) {
      const double inv_area_triangle = 1. / m->area_triangle[v];
      for (int k = 0; k < K; ++k) {
        double rvort = 0;
        for (int j = 0; j < 3; ++j) {
          const int je = m->edges_on_vertex[3 * v + j];
          rvort += m->dc_edge[je] * inv_area_triangle *
                   m->edge_sign_on_vertex[3 * v + j] *
                   md->vel_del2_edge[(size_t)je * K + k];
        }
        md->vel_del2_rvort_vertex[(size_t)v * K + k] = rvort;
      }
    }
    /* compute_vel_del2_div (vel_hyperdiff_edge.hpp:286-307) */
#pragma omp parallel for schedule(static)
    for (int c = 0; c < C; ++c) {
      const double inv_area_cell = 1. / m->area_cell[c];
      for (int k = 0; k < K; ++k) {
        double accum = 0;
        for (int j = 0; j < m->nedges_on_cell[c]; ++j) {
          const int je = m->edges_on_cell[6 * c + j];
          accum += m->dv_edge[je] * inv_area_cell *
                   m->edge_sign_on_cell[6 * c + j] *
                   md->vel_del2_edge[(size_t)je * K + k];
        }
        md->vel_del2_div_cell[(size_t)c * K + k] = accum;
      }
    }
  }

  /* compute_vtend (shallow_water_model.cpp:186-217): each enabled term adds
   * its own contribution to vn_tend in this order. */
#pragma omp parallel for schedule(static)
  for (int e = 0; e < E; ++e) {
    const int c0 = m->cells_on_edge[2 * e], c1 = m->cells_on_edge[2 * e + 1];
    const int v0 = m->vertices_on_edge[2 * e],
              v1 = m->vertices_on_edge[2 * e + 1];
    const double inv_dc = 1. / m->dc_edge[e];
    const double inv_dv = 1. / m->dv_edge[e];
    for (int k = 0; k < K; ++k) {
      const size_t i = (size_t)e * K + k;
      if (add_mode == 0)
        vn_tend[i] = 0;
      /* PotentialVortFluxOnEdge (pv_flux_edge.hpp:149-177) */
      if (md->en_pv) {
        double qt = 0;
        for (int j = 0; j < m->nedges_on_edge[e]; ++j) {
          const int je = m->edges_on_edge[12 * e + j];
          const size_t ij = (size_t)je * K + k;
          const double norm_vort =
              (md->norm_rvort_edge[i] + md->norm_pvort_edge[i] +
               md->norm_rvort_edge[ij] + md->norm_pvort_edge[ij]) *
              0.5;
          qt += m->weights_on_edge[12 * e + j] * md->flux_h_edge[ij] * vn[ij] *
                norm_vort;
        }
        vn_tend[i] += qt;
      }
      /* KineticEnergyGradOnEdge (ke_grad_edge.hpp:223-237) */
      if (md->en_ke)
        vn_tend[i] -= (md->ke_cell[(size_t)c1 * K + k] -
                       md->ke_cell[(size_t)c0 * K + k]) *
                      inv_dc;
      /* SSHGradOnEdge (ssh_grad_edge.hpp:281-294) */
      if (md->en_ssh)
        vn_tend[i] -= p->grav *
                      (h[(size_t)c1 * K + k] - h[(size_t)c0 * K + k]) * inv_dc;
      /* bottom drag, opt-in: the term commented out at
       * shallow_water_hierarchical.cpp:479-486 with h_drag_edge = h_mean
       * (:258-276) on the lowest level (max_level_edge_top = nlayers) */
      if (md->apply_drag && p->drag_coeff > 0 && k == K - 1) {
        const double inv_h_drag_edge = 1. / md->mean_h_edge[i];
        vn_tend[i] += -p->drag_coeff *
                      sqrt(md->ke_cell[(size_t)c0 * K + k] +
                           md->ke_cell[(size_t)c1 * K + k]) *
                      vn[i] * inv_h_drag_edge;
      }
      /* VelocityDiffusionOnEdge (vel_diff_edge.hpp:61-86) */
      if (md->en_vel_diff) {
        const double del2u =
            ((md->vel_div_cell[(size_t)c1 * K + k] -
              md->vel_div_cell[(size_t)c0 * K + k]) *
                 inv_dc -
             (md->rvort_vertex[(size_t)v1 * K + k] -
              md->rvort_vertex[(size_t)v0 * K + k]) *
                 inv_dv);
        vn_tend[i] += m->edge_mask[i] * p->visc_del2 *
                      m->mesh_scaling_del2[e] * del2u;
      }
      /* VelocityHyperDiffusionOnEdge::operator() (vel_hyperdiff_edge.hpp:309-334) */
      if (md->en_vel_hyperdiff) {
        const double del2u = ((md->vel_del2_div_cell[(size_t)c1 * K + k] -
                               md->vel_del2_div_cell[(size_t)c0 * K + k]) *
                                  inv_dc -
                              (md->vel_del2_rvort_vertex[(size_t)v1 * K + k] -
                               md->vel_del2_rvort_vertex[(size_t)v0 * K + k]) *
                                  inv_dv);
        vn_tend[i] -= m->edge_mask[i] * p->visc_del4 *
                      m->mesh_scaling_del4[e] * del2u;
      }
    }
  }
}

/* ShallowWaterModel::compute_tr_tendency (shallow_water_model.cpp:221-311).
 * The reference passes m_mean_h_edge as the flux thickness and
 * m_flux_h_edge as the mean thickness (:225-228); both hold the same values. */
void or_tr_tendency(or_model *md, double *tr_tend, const double *vn,
                    int add_mode) {
  const or_mesh *m = &md->m;
  const or_params *p = &md->p;
  const int K = m->nlayers, C = m->ncells, T = p->ntracers;
  const double *flux_h = md->mean_h_edge, *mean_h = md->flux_h_edge;
  const double *ntr = md->norm_tr_cell;

  if (md->en_tr_hyperdiff) {
    /* compute_tracer_del2 (tracer_hyperdiff_cell.hpp:301-336) */
#pragma omp parallel for collapse(2) schedule(static)
    for (int l = 0; l < T; ++l)
      for (int c = 0; c < C; ++c) {
        const double inv_area_cell = 1. / m->area_cell[c];
        for (int k = 0; k < K; ++k) {
          double del2 = 0;
          for (int j = 0; j < m->nedges_on_cell[c]; ++j) {
            const int je = m->edges_on_cell[6 * c + j];
            const double inv_dc_edge = 1. / m->dc_edge[je];
            const int c0 = m->cells_on_edge[2 * je], c1 = m->cells_on_edge[2 * je + 1];
            const double grad = (ntr[((size_t)l * C + c1) * K + k] -
                                 ntr[((size_t)l * C + c0) * K + k]) *
                                inv_dc_edge;
            del2 += m->dv_edge[je] * inv_area_cell *
                    m->edge_sign_on_cell[6 * c + j] *
                    mean_h[(size_t)je * K + k] * grad;
          }
          md->tracer_del2_cell[((size_t)l * C + c) * K + k] = del2;
        }
      }
  }

  const double *trd = md->tracer_del2_cell;
#pragma omp parallel for collapse(2) schedule(static)
  for (int l = 0; l < T; ++l)
    for (int c = 0; c < C; ++c) {
      const double inv_area_cell = 1. / m->area_cell[c];
      for (int k = 0; k < K; ++k) {
        const size_t i = ((size_t)l * C + c) * K + k;
        if (add_mode == 0)
          tr_tend[i] = 0;
        /* TracerHorzAdvOnCell (tracer_hadv_cell.hpp:60-90) */
        if (md->en_tr_hadv) {
          double accum = 0;
          for (int j = 0; j < m->nedges_on_cell[c]; ++j) {
            const int je = m->edges_on_cell[6 * c + j];
            const int c0 = m->cells_on_edge[2 * je], c1 = m->cells_on_edge[2 * je + 1];
            const double norm_tr_edge = (ntr[((size_t)l * C + c0) * K + k] +
                                         ntr[((size_t)l * C + c1) * K + k]) *
                                        0.5;
            accum -= m->dv_edge[je] * inv_area_cell *
                     m->edge_sign_on_cell[6 * c + j] *
                     flux_h[(size_t)je * K + k] * norm_tr_edge *
                     vn[(size_t)je * K + k];
          }
          tr_tend[i] += accum;
        }
        /* TracerDiffusionOnCell (tracer_diff_cell.hpp:162-193) */
        if (md->en_tr_diff) {
          double accum = 0;
          for (int j = 0; j < m->nedges_on_cell[c]; ++j) {
            const int je = m->edges_on_cell[6 * c + j];
            const double inv_dc_edge = 1. / m->dc_edge[je];
            const int c0 = m->cells_on_edge[2 * je], c1 = m->cells_on_edge[2 * je + 1];
            const double grad = (ntr[((size_t)l * C + c1) * K + k] -
                                 ntr[((size_t)l * C + c0) * K + k]) *
                                inv_dc_edge;
            accum += p->eddy_diff2 * inv_area_cell * m->dv_edge[je] *
                     m->edge_sign_on_cell[6 * c + j] *
                     mean_h[(size_t)je * K + k] * m->mesh_scaling_del2[je] *
                     grad;
          }
          tr_tend[i] += accum;
        }
        /* TracerHyperDiffusionOnCell::operator() (tracer_hyperdiff_cell.hpp:338-368) */
        if (md->en_tr_hyperdiff) {
          double accum = 0;
          for (int j = 0; j < m->nedges_on_cell[c]; ++j) {
            const int je = m->edges_on_cell[6 * c + j];
            const double inv_dc_edge = 1. / m->dc_edge[je];
            const int c0 = m->cells_on_edge[2 * je], c1 = m->cells_on_edge[2 * je + 1];
            const double grad = (trd[((size_t)l * C + c1) * K + k] -
                                 trd[((size_t)l * C + c0) * K + k]) *
                                inv_dc_edge;
            accum -= p->eddy_diff4 * inv_area_cell * m->dv_edge[je] *
                     m->edge_sign_on_cell[6 * c + j] *
                     m->mesh_scaling_del4[je] * grad;
          }
          tr_tend[i] += accum;
        }
      }
    }
}

/* LinearShallowWaterModel::compute_h_tendency / compute_vn_tendency
 * (shallow_water_hierarchical.cpp:680-740); f_edge = f0 (:15) */
static void linear_tendency(or_model *md, double *h_tend, double *vn_tend,
                            const double *h, const double *vn, int add_mode) {
  const or_mesh *m = &md->m;
  const int K = m->nlayers;
  if (!md->p.disable_h_tendency) {
#pragma omp parallel for schedule(static)
    for (int c = 0; c < m->ncells; ++c)
      for (int k = 0; k < K; ++k) {
        double accum = -0.0;
        for (int j = 0; j < m->nedges_on_cell[c]; ++j) {
          const int je = m->edges_on_cell[6 * c + j];
          accum += m->dv_edge[je] * m->edge_sign_on_cell[6 * c + j] *
                   vn[(size_t)je * K + k];
        }
        const double x = -md->h0 * accum / m->area_cell[c];
        if (add_mode == 1)
          h_tend[(size_t)c * K + k] += x;
        else
          h_tend[(size_t)c * K + k] = x;
      }
  }
  if (!md->p.disable_vn_tendency) {
#pragma omp parallel for schedule(static)
    for (int e = 0; e < m->nedges; ++e)
      for (int k = 0; k < K; ++k) {
        double vt = -0.0;
        for (int j = 0; j < m->nedges_on_edge[e]; ++j) {
          const int je = m->edges_on_edge[12 * e + j];
          vt += m->weights_on_edge[12 * e + j] * vn[(size_t)je * K + k];
        }
        const int c0 = m->cells_on_edge[2 * e], c1 = m->cells_on_edge[2 * e + 1];
        const double grad_h =
            (h[(size_t)c1 * K + k] - h[(size_t)c0 * K + k]) / m->dc_edge[e];
        const double x = md->p.f0 * vt - md->p.grav * grad_h;
        if (add_mode == 1)
          vn_tend[(size_t)e * K + k] += x;
        else
          vn_tend[(size_t)e * K + k] = x;
      }
  }
}

/* Setting a term member's m_enabled (terms numbered as in
 * shallow_water_model.hpp:19-29). */
int or_model_set_term(or_model *md, int term, int enabled) {
  int *f[9] = {&md->en_hadv, &md->en_pv, &md->en_ke, &md->en_ssh,
               &md->en_vel_diff, &md->en_vel_hyperdiff, &md->en_tr_hadv,
               &md->en_tr_diff, &md->en_tr_hyperdiff};
  if (term < 0 || term > 8)
    return 1;
  *f[term] = enabled != 0;
  return 0;
}

void or_compute_tendency(or_model *md, double *h_tend, double *vn_tend,
                         double *tr_tend, const double *h, const double *vn,
                         const double *tr, double t, int add_mode) {
  (void)t; /* only the additional_tendency hook (not modelled) reads t */
  if (md->linear) {
    linear_tendency(md, h_tend, vn_tend, h, vn, add_mode);
    return;
  }
  or_aux_compute(md, h, vn, tr);
  if (!md->p.disable_h_tendency)
    or_h_tendency(md, h_tend, vn, add_mode);
  if (!md->p.disable_vn_tendency)
    or_vn_tendency(md, vn_tend, h, vn, add_mode);
  if (md->p.ntracers > 0)
    or_tr_tendency(md, tr_tend, vn, add_mode);
}

/* ------------------------------------------------------------ steppers --- */

static void ensure_stepper(or_model *md, int kind, int nstages) {
  if (md->st_kind == kind && md->st_nstages == nstages)
    return;
  free(md->st_tend);
  free(md->st_provis);
  free(md->st_old);
  const size_t K = md->m.nlayers;
  const size_t n = (md->m.ncells + md->m.nedges +
                    (size_t)md->p.ntracers * md->m.ncells) * K;
  /* LSRKStepper ctor zeroes m_tend (lsrk.cpp:8-13); RK4's views are
   * zero-initialised too. */
  md->st_tend = zalloc(n);
  md->st_provis = kind == 0 ? zalloc(n) : NULL;
  md->st_old = kind == 0 ? zalloc(n) : NULL;
  md->st_kind = kind;
  md->st_nstages = nstages;
}

/* axpy over one field in the reference's form y (+)= (dt * b) * x */
static void acc_field(double *y, const double *x, double a, size_t n) {
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < n; ++i)
    y[i] += a * x[i];
}

int or_step(or_model *md, int kind, int nstages, double *h, double *vn,
            double *tr, double t0, double dt, int nsteps) {
  const size_t K = md->m.nlayers, C = md->m.ncells, E = md->m.nedges;
  const size_t T = md->p.ntracers;
  const size_t nh = C * K, nv = E * K, nt = T * C * K;
  if (kind == 1 && nstages != 5 && nstages != 1)
    return 1;
  ensure_stepper(md, kind, nstages);
  double *th = md->st_tend, *tv = th + nh, *tt = tv + nv;

  for (int s = 0; s < nsteps; ++s) {
    const double t = t0 + s * dt;
    if (kind == 0) {
      /* RK4Stepper::do_step (rk4.cpp:28-104), coefficients rk4.cpp:14-25 */
      static const double rka[3] = {1. / 2, 1. / 2, 1};
      static const double rkb[4] = {1. / 6, 1. / 3, 1. / 3, 1. / 6};
      static const double rkc[3] = {1. / 2, 1. / 2, 1};
      double *ph = md->st_provis, *pv = ph + nh, *pt = pv + nv;
      double *oh = md->st_old, *ov = oh + nh, *ot = ov + nv;
      memcpy(oh, h, nh * 8);
      memcpy(ov, vn, nv * 8);
      if (T)
        memcpy(ot, tr, nt * 8);
      or_compute_tendency(md, th, tv, tt, h, vn, tr, t, 0);
      for (int stage = 0; stage < 4; ++stage) {
        const double rkb_stage = rkb[stage];
        acc_field(h, th, dt * rkb_stage, nh);
        acc_field(vn, tv, dt * rkb_stage, nv);
        if (T)
          acc_field(tr, tt, dt * rkb_stage, nt);
        if (stage < 3) {
          const double stagetime = t + rkc[stage] * dt;
          const double a = dt * rka[stage];
#pragma omp parallel for schedule(static)
          for (size_t i = 0; i < nh; ++i)
            ph[i] = oh[i] + a * th[i];
#pragma omp parallel for schedule(static)
          for (size_t i = 0; i < nv; ++i)
            pv[i] = ov[i] + a * tv[i];
#pragma omp parallel for schedule(static)
          for (size_t i = 0; i < nt; ++i)
            pt[i] = ot[i] + a * tt[i];
          or_compute_tendency(md, th, tv, tt, ph, pv, pt, stagetime, 0);
        }
      }
    } else {
      /* LSRKStepper::do_step (lsrk.cpp:36-89), coefficients lsrk.cpp:16-33 */
      static const double rka5[5] = {0., -567301805773. / 1357537059087.,
                                     -2404267990393. / 2016746695238.,
                                     -3550918686646. / 2091501179385.,
                                     -1275806237668. / 842570457699.};
      static const double rkb5[5] = {1432997174477. / 9575080441755.,
                                     5161836677717. / 13612068292357.,
                                     1720146321549. / 2090206949498.,
                                     3134564353537. / 4481467310338.,
                                     2277821191437. / 14882151754819.};
      static const double rkc5[5] = {0., 1432997174477. / 9575080441755.,
                                     2526269341429. / 6820363962896.,
                                     2006345519317. / 3224310063776.,
                                     2802321613138. / 2924317926251.};
      static const double rka1[1] = {0}, rkb1[1] = {1}, rkc1[1] = {0};
      const double *rka = nstages == 5 ? rka5 : rka1;
      const double *rkb = nstages == 5 ? rkb5 : rkb1;
      const double *rkc = nstages == 5 ? rkc5 : rkc1;
      for (int stage = 0; stage < nstages; ++stage) {
        const double rka_stage = rka[stage];
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < nh; ++i)
          th[i] *= rka_stage;
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < nv; ++i)
          tv[i] *= rka_stage;
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < nt; ++i)
          tt[i] *= rka_stage;
        const double stagetime = t + rkc[stage] * dt;
        or_compute_tendency(md, th, tv, tt, h, vn, tr, stagetime, 1);
        const double rkb_stage = rkb[stage];
        acc_field(h, th, dt * rkb_stage, nh);
        acc_field(vn, tv, dt * rkb_stage, nv);
        if (T)
          acc_field(tr, tt, dt * rkb_stage, nt);
      }
    }
  }
  return 0;
}

/* --------------------------------------------------------- diagnostics --- */

/* energy_integral (shallow_water_diagnostics.cpp:5-38) */
double or_energy_integral(or_model *md, const double *h, const double *vn) {
  const or_mesh *m = &md->m;
  const int K = m->nlayers;
  double total = 0;
  for (int c = 0; c < m->ncells; ++c)
    for (int k = 0; k < (m->max_level_cell ? m->max_level_cell[c] : K); ++k) {
      double KE = 0;
      for (int j = 0; j < m->nedges_on_cell[c]; ++j) {
        const int je = m->edges_on_cell[6 * c + j];
        const double area_edge = m->dv_edge[je] * m->dc_edge[je];
        const double u = vn[(size_t)je * K + k];
        KE += area_edge * u * u / 4;
      }
      KE /= m->area_cell[c];
      const double hc = h[(size_t)c * K + k];
      /* the linear model weights KE by h0
       * (shallow_water_hierarchical.cpp:743-771) */
      total += m->area_cell[c] *
               (md->p.grav * hc * hc / 2 + (md->linear ? md->h0 : hc) * KE);
    }
  return total;
}

/* mass_integral (shallow_water_diagnostics.cpp:40-58) */
double or_mass_integral(or_model *md, const double *h) {
  const or_mesh *m = &md->m;
  const int K = m->nlayers;
  double total = 0;
  for (int c = 0; c < m->ncells; ++c)
    for (int k = 0; k < (m->max_level_cell ? m->max_level_cell[c] : K); ++k)
      total += m->area_cell[c] * h[(size_t)c * K + k];
  return total;
}

/* circulation_integral (shallow_water_diagnostics.cpp:60-89) */
double or_circulation_integral(or_model *md, const double *vn) {
  const or_mesh *m = &md->m;
  const int K = m->nlayers;
  double total = 0;
  for (int v = 0; v < m->nvertices; ++v)
    for (int k = 0;
         k < (m->max_level_vertex_bot ? m->max_level_vertex_bot[v] : K); ++k) {
      double cir = -0.0;
      for (int j = 0; j < 3; ++j) {
        const int je = m->edges_on_vertex[3 * v + j];
        cir += m->dc_edge[je] * m->edge_sign_on_vertex[3 * v + j] *
               vn[(size_t)je * K + k];
      }
      total += cir + md->f_vertex[v] * m->area_triangle[v];
    }
  return total;
}
