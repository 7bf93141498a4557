// Convergence of the mesh operators on the drop-in mesh (re-hosts
// test/operator_convergence.cpp): gradient, divergence and TRiSK tangential
// reconstruction at rate 2, curl at rate 1 (L-infinity, +-0.05), nx = 6..96.
// The tables come from the library's mesh builder; the operators are
// evaluated on the host from those tables as in the reference test.
#include <omega_gpu.hpp>

#include <algorithm>
#include <cstdio>

using namespace omega;

int main() {
  Real err[4][5];
  Int nx = 6;
  for (Int l = 0; l < 5; ++l, nx *= 2) {
    PlanarHexagonalMesh m(nx, nx);
    const Real Lx = m.m_period_x, Ly = m.m_period_y, tw = 2 * pi;
    std::vector<Real> f(m.m_ncells), u(m.m_nedges);
    for (Int c = 0; c < m.m_ncells; ++c)
      f[c] = std::sin(tw * m.m_x_cell[c] / Lx) * std::sin(tw * m.m_y_cell[c] / Ly);
    Real eg = 0, ed = 0, ec = 0, er = 0;
    for (Int e = 0; e < m.m_nedges; ++e) {
      const Real x = m.m_x_edge[e], y = m.m_y_edge[e];
      const Real nxv = std::cos(m.m_angle_edge[e]), nyv = std::sin(m.m_angle_edge[e]);
      const Real vx = std::sin(tw * x / Lx) * std::cos(tw * y / Ly);
      const Real vy = std::cos(tw * x / Lx) * std::sin(tw * y / Ly);
      u[e] = nxv * vx + nyv * vy;
      const Int c0 = m.m_cells_on_edge[2 * e], c1 = m.m_cells_on_edge[2 * e + 1];
      const Real grad = (f[c1] - f[c0]) / m.m_dc_edge[e];
      const Real gx = tw / Lx * std::cos(tw * x / Lx) * std::sin(tw * y / Ly);
      const Real gy = tw / Ly * std::sin(tw * x / Lx) * std::cos(tw * y / Ly);
      eg = std::max(eg, std::abs(nxv * gx + nyv * gy - grad));
    }
    for (Int e = 0; e < m.m_nedges; ++e) {
      const Real x = m.m_x_edge[e], y = m.m_y_edge[e];
      const Real nxv = std::cos(m.m_angle_edge[e]), nyv = std::sin(m.m_angle_edge[e]);
      const Real vx = std::sin(tw * x / Lx) * std::cos(tw * y / Ly);
      const Real vy = std::cos(tw * x / Lx) * std::sin(tw * y / Ly);
      Real rec = 0;
      for (Int j = 0; j < m.m_nedges_on_edge[e]; ++j)
        rec += m.m_weights_on_edge[12 * e + j] * u[m.m_edges_on_edge[12 * e + j]];
      er = std::max(er, std::abs(-nyv * vx + nxv * vy - rec));
    }
    for (Int c = 0; c < m.m_ncells; ++c) {
      Real acc = 0;
      for (Int j = 0; j < m.m_nedges_on_cell[c]; ++j) {
        const Int e = m.m_edges_on_cell[6 * c + j];
        acc += m.m_dv_edge[e] * m.m_edge_sign_on_cell[6 * c + j] * u[e];
      }
      const Real x = m.m_x_cell[c], y = m.m_y_cell[c];
      const Real ex = tw * (1. / Lx + 1. / Ly) * std::cos(tw * x / Lx) * std::cos(tw * y / Ly);
      ed = std::max(ed, std::abs(ex - acc / m.m_area_cell[c]));
    }
    for (Int v = 0; v < m.m_nvertices; ++v) {
      Real acc = 0;
      for (Int j = 0; j < 3; ++j) {
        const Int e = m.m_edges_on_vertex[3 * v + j];
        acc += m.m_dc_edge[e] * m.m_edge_sign_on_vertex[3 * v + j] * u[e];
      }
      const Real x = m.m_x_vertex[v], y = m.m_y_vertex[v];
      const Real ex = tw * (-1. / Lx + 1. / Ly) * std::sin(tw * x / Lx) * std::sin(tw * y / Ly);
      ec = std::max(ec, std::abs(ex - acc / m.m_area_triangle[v]));
    }
    err[0][l] = eg;
    err[1][l] = ed;
    err[2][l] = ec;
    err[3][l] = er;
  }
  const char *names[4] = {"Gradient", "Divergence", "Curl", "Reconstruction"};
  const Real expect[4] = {2, 2, 1, 2};
  int rc = 0;
  for (int o = 0; o < 4; ++o) {
    std::printf("%s convergence\n", names[o]);
    for (int l = 0; l < 5; ++l) {
      if (l == 0)
        std::printf("%d %.9g\n", l, err[o][l]);
      else
        std::printf("%d %.9g %.6f\n", l, err[o][l], std::log2(err[o][l - 1] / err[o][l]));
    }
    const Real rate = std::log2(err[o][3] / err[o][4]);
    if (!(std::abs(rate - expect[o]) < 0.05)) {
      std::printf("FAIL: %s rate %.4f\n", names[o], rate);
      rc = 1;
    }
  }
  return rc;
}
