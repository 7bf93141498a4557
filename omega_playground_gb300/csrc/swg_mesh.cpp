// Host construction of the doubly periodic planar hexagonal MPAS mesh.
//
// Produces the same tables, bit for bit, as omega_playground's
// PlanarHexagonalMesh (src/mesh/planar_hexagonal_mesh.cpp:8-398) followed by
// MPASMesh::finalize_mesh (src/mesh/mpas_mesh.cpp:5-57):
//  - cells are numbered row-major, cell c owns edges 3c..3c+2 (west,
//    south-west, south-east faces) and vertices 2c, 2c+1;
//  - odd rows are shifted half a cell east;
//  - the TRiSK weights of the regular hexagon are +-1/3, +-1/6, 0 (times
//    1/sqrt(3)), listed for the five other edges of each adjacent cell.
// The floating-point expressions keep the reference's association so the
// geometry is bit-identical.  Cells are visited in the reference's MDRange
// order (row outer, column inner); for odd ny, where the reference's
// parallel loop writes some slots twice, this keeps the serial last writer.
#include "swg_internal.h"

#include <cmath>
#include <cstring>

namespace swg {
namespace {

struct HexGrid {
  int nx, ny;
  int cell(int col, int row) const { return row * nx + col; }
  // neighbour nb (0..5) of (col,row), counter-clockwise starting west
  int neighbour(int col, int row, int nb) const {
    // column offsets for even and odd rows, row offsets (both rows)
    static const int dcol_even[6] = {-1, -1, 0, 1, 0, -1};
    static const int dcol_odd[6] = {-1, 0, 1, 1, 1, 0};
    static const int drow[6] = {0, -1, -1, 0, 1, 1};
    const int dc = (row % 2 == 0) ? dcol_even[nb] : dcol_odd[nb];
    int c = col + dc, r = row + drow[nb];
    c = c < 0 ? nx - 1 : (c >= nx ? 0 : c);
    r = r < 0 ? ny - 1 : (r >= ny ? 0 : r);
    return cell(c, r);
  }
  int edge(int c, int col, int row, int nb) const {
    return nb < 3 ? 3 * c + nb : 3 * neighbour(col, row, nb) + (nb - 3);
  }
  int vertex(int c, int col, int row, int nb) const {
    switch (nb) {
    case 0: return 2 * c;
    case 1: return 2 * c + 1;
    case 2: return 2 * neighbour(col, row, 2);
    case 3: return 2 * neighbour(col, row, 3) + 1;
    case 4: return 2 * neighbour(col, row, 3);
    default: return 2 * neighbour(col, row, 4) + 1;
    }
  }
};

} // namespace

int build_planar_hex(int nx, int ny, double dc, swg_hex_tables *t,
                     double *period_x, double *period_y) {
  if (nx < 1 || ny < 1)
    return fail(SWG_ERR_ARG, "planar hex mesh needs nx >= 1 and ny >= 1");
  if ((long long)nx * ny * 3 > 0x7fffffffLL)
    return fail(SWG_ERR_ARG, "planar hex mesh too large for int32 indices");
  const HexGrid g{nx, ny};
  const int C = nx * ny, E = 3 * C, V = 2 * C;
  const double s3 = std::sqrt(3.0);
  const double pi = 3.14159265358979323846; // omega::pi (M_PI)
  if (period_x)
    *period_x = nx * dc;
  if (period_y)
    *period_y = ny * dc * s3 / 2;

  // work arrays (the caller may skip any output table)
  std::vector<int> eoc(6 * C), voc(6 * C), coc(6 * C), coe(2 * E, 0),
      voe(2 * E, 0), eoe(12 * E, 0), cov(3 * V, 0), eov(3 * V, 0);
  std::vector<double> woe(12 * E, 0.0);

  static const double w_ccw[3][5] = {{1. / 3, 1. / 6, 0, 1. / 6, 1. / 3},
                                     {1. / 3, -1. / 6, 0, 1. / 6, -1. / 3},
                                     {-1. / 3, -1. / 6, 0, -1. / 6, -1. / 3}};
  for (int row = 0; row < ny; ++row) {
    for (int col = 0; col < nx; ++col) {
      const int c = g.cell(col, row);
      int *ce = &eoc[6 * c], *cv = &voc[6 * c];
      for (int j = 0; j < 6; ++j) {
        coc[6 * c + j] = g.neighbour(col, row, j);
        ce[j] = g.edge(c, col, row, j);
        cv[j] = g.vertex(c, col, row, j);
      }
      for (int j = 0; j < 3; ++j)
        coe[2 * ce[j] + 1] = c;
      for (int j = 3; j < 6; ++j)
        coe[2 * ce[j] + 0] = c;
      for (int j = 0; j < 3; ++j) {
        voe[2 * ce[j] + 0] = cv[j + 1];
        voe[2 * ce[j] + 1] = cv[j];
      }
      // edges 3..5 list the cell's other edges in slots 0-4, edges 0..2 in
      // slots 5-9, both counter-clockwise from the next edge
      for (int i = 3; i < 6; ++i)
        for (int s = 0; s < 5; ++s)
          eoe[12 * ce[i] + s] = ce[(i + 1 + s) % 6];
      for (int i = 0; i < 3; ++i)
        for (int s = 0; s < 5; ++s)
          eoe[12 * ce[i] + 5 + s] = ce[(i + 1 + s) % 6];
      for (int i = 0; i < 3; ++i)
        for (int s = 0; s < 5; ++s) {
          woe[12 * ce[3 + i] + s] = w_ccw[i][s];
          woe[12 * ce[i] + 5 + s] = w_ccw[i][s];
        }
      cov[3 * cv[1] + 2] = c;
      cov[3 * cv[3] + 0] = c;
      cov[3 * cv[5] + 1] = c;
      cov[3 * cv[0] + 0] = c;
      cov[3 * cv[2] + 1] = c;
      cov[3 * cv[4] + 2] = c;
      eov[3 * cv[0] + 0] = ce[0];
      eov[3 * cv[1] + 0] = ce[0];
      eov[3 * cv[2] + 2] = ce[1];
      eov[3 * cv[1] + 2] = ce[1];
      eov[3 * cv[2] + 1] = ce[2];
      eov[3 * cv[3] + 1] = ce[2];
    }
  }
  for (auto &w : woe)
    w *= 1. / std::sqrt(3.0);

  auto put_i = [](int *dst, const std::vector<int> &src) {
    if (dst)
      std::memcpy(dst, src.data(), src.size() * sizeof(int));
  };
  put_i(t->edges_on_cell, eoc);
  put_i(t->vertices_on_cell, voc);
  put_i(t->cells_on_cell, coc);
  put_i(t->cells_on_edge, coe);
  put_i(t->vertices_on_edge, voe);
  put_i(t->edges_on_edge, eoe);
  put_i(t->cells_on_vertex, cov);
  put_i(t->edges_on_vertex, eov);
  if (t->weights_on_edge)
    std::memcpy(t->weights_on_edge, woe.data(), woe.size() * sizeof(double));
  if (t->nedges_on_cell)
    for (int c = 0; c < C; ++c)
      t->nedges_on_cell[c] = 6;
  if (t->nedges_on_edge)
    for (int e = 0; e < E; ++e)
      t->nedges_on_edge[e] = 10;

  // geometry (planar_hexagonal_mesh.cpp:329-395)
  std::vector<double> xc(C), yc(C);
  for (int row = 0; row < ny; ++row)
    for (int col = 0; col < nx; ++col) {
      const int c = g.cell(col, row);
      xc[c] = (row % 2 == 0) ? dc * col + dc / 2 : dc * (col + 1);
      yc[c] = dc * (row + 1) * s3 / 2;
      if (t->area_cell)
        t->area_cell[c] = dc * dc * s3 / 2;
      const int *ce = &eoc[6 * c], *cv = &voc[6 * c];
      if (t->x_edge) {
        t->x_edge[ce[0]] = xc[c] - dc / 2;
        t->x_edge[ce[1]] = xc[c] - dc / 2 * std::cos(pi / 3);
        t->x_edge[ce[2]] = xc[c] + dc / 2 * std::cos(pi / 3);
      }
      if (t->y_edge) {
        t->y_edge[ce[0]] = yc[c];
        t->y_edge[ce[1]] = yc[c] - dc / 2 * std::sin(pi / 3);
        t->y_edge[ce[2]] = yc[c] - dc / 2 * std::sin(pi / 3);
      }
      if (t->angle_edge) {
        t->angle_edge[ce[0]] = 0;
        t->angle_edge[ce[1]] = pi / 3;
        t->angle_edge[ce[2]] = 2 * pi / 3;
      }
      if (t->x_vertex) {
        t->x_vertex[cv[0]] = xc[c] - dc / 2;
        t->x_vertex[cv[1]] = xc[c] - dc / 2;
      }
      if (t->y_vertex) {
        t->y_vertex[cv[0]] = yc[c] + dc * s3 / 6;
        t->y_vertex[cv[1]] = yc[c] - dc * s3 / 6;
      }
    }
  if (t->x_cell)
    std::memcpy(t->x_cell, xc.data(), C * sizeof(double));
  if (t->y_cell)
    std::memcpy(t->y_cell, yc.data(), C * sizeof(double));
  for (int e = 0; e < E; ++e) {
    if (t->dc_edge)
      t->dc_edge[e] = dc;
    if (t->dv_edge)
      t->dv_edge[e] = dc * s3 / 3;
  }
  for (int v = 0; v < V; ++v) {
    if (t->area_triangle)
      t->area_triangle[v] = dc * dc * s3 / 4;
    if (t->kiteareas_on_vertex)
      for (int j = 0; j < 3; ++j)
        t->kiteareas_on_vertex[3 * v + j] = dc * dc * s3 / 12;
  }

  // finalize_mesh (mpas_mesh.cpp:21-46)
  for (int c = 0; c < C; ++c)
    for (int j = 0; j < 6; ++j) {
      if (t->edge_sign_on_cell)
        t->edge_sign_on_cell[6 * c + j] = coe[2 * eoc[6 * c + j]] == c ? 1 : -1;
      if (t->kite_index_on_cell) {
        int idx = 0;
        const int jv = voc[6 * c + j];
        for (int l = 0; l < 3; ++l)
          if (cov[3 * jv + l] == c)
            idx = l;
        t->kite_index_on_cell[6 * c + j] = idx;
      }
    }
  if (t->edge_sign_on_vertex)
    for (int v = 0; v < V; ++v)
      for (int j = 0; j < 3; ++j)
        t->edge_sign_on_vertex[3 * v + j] =
            voe[2 * eov[3 * v + j]] == v ? -1 : 1;
  return SWG_OK;
}

} // namespace swg

extern "C" int swg_planar_hex_mesh_build(int nx, int ny, double dc,
                                         swg_hex_tables *out,
                                         double *period_x,
                                         double *period_y) try {
  if (!out)
    return swg::fail(SWG_ERR_ARG, "swg_planar_hex_mesh_build: out is NULL");
  return swg::build_planar_hex(nx, ny, dc, out, period_x, period_y);
} SWG_ABI_CATCH("swg_planar_hex_mesh_build")
