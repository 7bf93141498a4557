// The reference benchmark driver on the GB300 path (re-hosts
// benchmark/benchmark.cpp): double-vortex initial state, every dissipation
// term switched on at 1e-5, 5-stage LSRK (1-stage when nsteps == 1), one
// untimed warm-up step, then `nsteps` timed steps between fences.
//   usage: benchmark [nx=64] [nlayers=64] [ntracers=1] [nsteps=10]
// Prints the loop's wall seconds to stderr (as the reference does) and a
// summary line with cell-level-stage updates per second to stdout.
#include <omega_gpu.hpp>

#include <chrono>
#include <cstdio>
#include <memory>
#include <string>

using namespace omega;

struct DoubleVortex {
  Real m_g = 9.80616, m_lx = 5000000, m_ly = 5000000 * std::sqrt(3) / 2;
  Real m_coriolis = 0.00006147, m_h0 = 750, m_ox = 0.1, m_oy = 0.1;
  Real m_sigmax = 3. / 40. * m_lx, m_sigmay = 3. / 40. * m_ly, m_dh = 75;
  Real m_xc1 = (0.5 - m_ox) * m_lx, m_yc1 = (0.5 - m_oy) * m_ly;
  Real m_xc2 = (0.5 + m_ox) * m_lx, m_yc2 = (0.5 + m_oy) * m_ly;
  void primes(Real x, Real y, Real &x1, Real &y1, Real &x2, Real &y2) const {
    x1 = m_lx / (pi * m_sigmax) * std::sin(pi / m_lx * (x - m_xc1));
    y1 = m_ly / (pi * m_sigmay) * std::sin(pi / m_ly * (y - m_yc1));
    x2 = m_lx / (pi * m_sigmax) * std::sin(pi / m_lx * (x - m_xc2));
    y2 = m_ly / (pi * m_sigmay) * std::sin(pi / m_ly * (y - m_yc2));
  }
  Real h(Real x, Real y) const {
    Real x1, y1, x2, y2;
    primes(x, y, x1, y1, x2, y2);
    return m_h0 - m_dh * (std::exp(-0.5 * (x1 * x1 + y1 * y1)) +
                          std::exp(-0.5 * (x2 * x2 + y2 * y2)) -
                          4. * pi * m_sigmax * m_sigmay / m_lx / m_ly);
  }
  Real vx(Real x, Real y) const {
    Real x1, y1, x2, y2;
    primes(x, y, x1, y1, x2, y2);
    const Real a = m_ly / (2.0 * pi * m_sigmay) * std::sin(2.0 * pi / m_ly * (y - m_yc1));
    const Real b = m_ly / (2.0 * pi * m_sigmay) * std::sin(2.0 * pi / m_ly * (y - m_yc2));
    return -m_g * m_dh / m_coriolis / m_sigmay *
           (a * std::exp(-0.5 * (x1 * x1 + y1 * y1)) + b * std::exp(-0.5 * (x2 * x2 + y2 * y2)));
  }
  Real vy(Real x, Real y) const {
    Real x1, y1, x2, y2;
    primes(x, y, x1, y1, x2, y2);
    const Real a = m_lx / (2.0 * pi * m_sigmax) * std::sin(2.0 * pi / m_lx * (x - m_xc1));
    const Real b = m_lx / (2.0 * pi * m_sigmax) * std::sin(2.0 * pi / m_lx * (x - m_xc2));
    return m_g * m_dh / m_coriolis / m_sigmax *
           (a * std::exp(-0.5 * (x1 * x1 + y1 * y1)) + b * std::exp(-0.5 * (x2 * x2 + y2 * y2)));
  }
};

int main(int argc, char **argv) {
  const Int nx = argc > 1 ? std::stoi(argv[1]) : 64;
  const Int nlayers = argc > 2 ? std::stoi(argv[2]) : 64;
  const Int ntracers = argc > 3 ? std::stoi(argv[3]) : 1;
  const Int nsteps = argc > 4 ? std::stoi(argv[4]) : 10;
  DoubleVortex dv;
  auto mesh = std::make_unique<PlanarHexagonalMesh>(nx, nx, dv.m_lx / nx, nlayers);
  ShallowWaterParams params;
  params.m_ntracers = ntracers;
  params.m_f0 = dv.m_coriolis;
  params.m_grav = dv.m_g;
  params.m_visc_del2 = 1e-5;
  params.m_visc_del4 = 1e-5;
  params.m_eddy_diff2 = 1e-5;
  params.m_eddy_diff4 = 1e-5;
  ShallowWaterModel model(mesh.get(), params);
  ShallowWaterState state(mesh.get(), params);
  LSRKStepper stepper(model, nsteps == 1 ? 1 : 5);
  const Real dt = 0.1 * mesh->m_dc / std::sqrt(params.m_grav * dv.m_h0);
  const Int K = nlayers, C = mesh->m_ncells, E = mesh->m_nedges;
  std::vector<Real> h(size_t(C) * K), vn(size_t(E) * K),
      tr(size_t(ntracers) * C * K, 1000.0);
  for (Int c = 0; c < C; ++c)
    for (Int k = 0; k < K; ++k)
      h[size_t(c) * K + k] = dv.h(mesh->m_x_cell[c], mesh->m_y_cell[c]);
  for (Int e = 0; e < E; ++e) {
    const Real x = mesh->m_x_edge[e], y = mesh->m_y_edge[e];
    const Real u = std::cos(mesh->m_angle_edge[e]) * dv.vx(x, y) +
                   std::sin(mesh->m_angle_edge[e]) * dv.vy(x, y);
    for (Int k = 0; k < K; ++k)
      vn[size_t(e) * K + k] = u;
  }
  state.upload(h, vn, tr);
  stepper.do_step(0, dt, state);
  fence();
  const auto ts = std::chrono::steady_clock::now();
  for (Int step = 0; step < nsteps; ++step)
    stepper.do_step((step + 1) * dt, dt, state);
  fence();
  const auto te = std::chrono::steady_clock::now();
  const double sec = std::chrono::duration<double>(te - ts).count();
  std::fprintf(stderr, "%g\n", sec);
  const Int stages = nsteps == 1 ? 1 : 5;
  std::printf("benchmark nx=%d nlayers=%d ntracers=%d nsteps=%d seconds=%.6f "
              "updates_per_s=%.6e\n", nx, nlayers, ntracers, nsteps, sec,
              double(C) * K * stages * nsteps / sec);
  return 0;
}
