// Double-vortex conservation test on the GB300 path (re-hosts
// test/double_vortex.cpp): nx = 25 with ny = ceil(Ly / (dc sqrt(3)/2)) = 29
// (odd), 5-stage LSRK, cfl 0.1, 2e5 s, no dissipation; relative change of
// mass and circulation < 5e-14 and of energy < 1e-10.
#include <omega_gpu.hpp>

#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>

using namespace omega;

struct DoubleVortex {
  Real m_g = 9.80616, m_lx = 5000000, m_ly = 5000000, m_coriolis = 0.00006147;
  Real m_h0 = 750, m_ox = 0.1, m_oy = 0.1;
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
    const Real yy1 = m_ly / (2.0 * pi * m_sigmay) * std::sin(2.0 * pi / m_ly * (y - m_yc1));
    const Real yy2 = m_ly / (2.0 * pi * m_sigmay) * std::sin(2.0 * pi / m_ly * (y - m_yc2));
    return -m_g * m_dh / m_coriolis / m_sigmay *
           (yy1 * std::exp(-0.5 * (x1 * x1 + y1 * y1)) +
            yy2 * std::exp(-0.5 * (x2 * x2 + y2 * y2)));
  }
  Real vy(Real x, Real y) const {
    Real x1, y1, x2, y2;
    primes(x, y, x1, y1, x2, y2);
    const Real xx1 = m_lx / (2.0 * pi * m_sigmax) * std::sin(2.0 * pi / m_lx * (x - m_xc1));
    const Real xx2 = m_lx / (2.0 * pi * m_sigmax) * std::sin(2.0 * pi / m_lx * (x - m_xc2));
    return m_g * m_dh / m_coriolis / m_sigmax *
           (xx1 * std::exp(-0.5 * (x1 * x1 + y1 * y1)) +
            xx2 * std::exp(-0.5 * (x2 * x2 + y2 * y2)));
  }
};

int main(int argc, char **argv) {
  DoubleVortex dv;
  const Int nx = argc > 1 ? std::stoi(argv[1]) : 25;
  const Real cfl = argc > 2 ? std::stod(argv[2]) : 0.1;
  const Real dc = dv.m_lx / nx;
  const Int ny = Int(std::ceil(dv.m_ly / (dc * std::sqrt(3) / 2)));
  auto mesh = std::make_unique<PlanarHexagonalMesh>(nx, ny, dc);
  ShallowWaterParams params;
  params.m_f0 = dv.m_coriolis;
  params.m_grav = dv.m_g;
  ShallowWaterModel model(mesh.get(), params);
  ShallowWaterState state(mesh.get(), params);
  LSRKStepper stepper(model);
  const Real timeend = 200 * 1000;
  Real dt = cfl * mesh->m_dc / std::sqrt(params.m_grav * dv.m_h0);
  const Int nsteps = Int(std::ceil(timeend / dt));
  dt = timeend / nsteps;
  const Int K = mesh->m_nlayers;
  std::vector<Real> h(size_t(mesh->m_ncells) * K), vn(size_t(mesh->m_nedges) * K);
  for (Int c = 0; c < mesh->m_ncells; ++c)
    for (Int k = 0; k < K; ++k)
      h[c * K + k] = dv.h(mesh->m_x_cell[c], mesh->m_y_cell[c]);
  for (Int e = 0; e < mesh->m_nedges; ++e)
    for (Int k = 0; k < K; ++k) {
      const Real x = mesh->m_x_edge[e], y = mesh->m_y_edge[e];
      vn[e * K + k] = std::cos(mesh->m_angle_edge[e]) * dv.vx(x, y) +
                      std::sin(mesh->m_angle_edge[e]) * dv.vy(x, y);
    }
  state.upload(h, vn);
  const Real mass0 = mass_integral(state, model);
  const Real cir0 = circulation_integral(state, model);
  const Real en0 = energy_integral(state, model);
  for (Int step = 0; step < nsteps; ++step)
    stepper.do_step(step * dt, dt, state);
  const Real dm = (mass_integral(state, model) - mass0) / mass0;
  const Real dcir = (circulation_integral(state, model) - cir0) / cir0;
  const Real den = (energy_integral(state, model) - en0) / en0;
  std::printf("Mesh %dx%d, %d steps\nMass change: %.6g\nCirculation change: "
              "%.6g\nEnergy change: %.6g\n", nx, ny, nsteps, dm, dcir, den);
  if (std::abs(dm) > 5e-14 || std::abs(dcir) > 5e-14 || std::abs(den) > 1e-10) {
    std::printf("FAIL: conservation bound exceeded\n");
    return 1;
  }
  return 0;
}
