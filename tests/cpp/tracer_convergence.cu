// Tracer convergence tests on the GB300 path (re-hosts
// test/tracer_advection_convergence.cpp, tracer_diffusion_convergence.cpp and
// tracer_hyperdiffusion_convergence.cpp): thickness and velocity frozen
// (disable_h/vn_tendency), one tracer, 5-stage LSRK, L2 error against the
// exact solution on two meshes, rate 2 +- 0.05.
//   usage: tracer_convergence advection|diffusion|hyperdiffusion
#include <omega_gpu.hpp>

#include <cstdio>
#include <cstring>
#include <memory>

using namespace omega;

struct Case {
  int kind; // 0 advection, 1 diffusion, 2 hyperdiffusion
  Real lx, ly, kappa;
  Real h(Real x, Real) const {
    return kind == 0 ? std::exp(std::cos(2 * pi * x / lx)) : 1.0;
  }
  Real tr(Real x, Real y, Real t) const {
    if (kind == 0)
      return std::sin(2 * pi * (x - t) / lx) * std::sin(2 * pi * (y - t) / ly);
    const Real c = 4 * pi * pi * (1. / (lx * lx) + 1. / (ly * ly));
    const Real decay = kind == 1 ? std::exp(-kappa * c * t)
                                 : std::exp(-kappa * c * c * t);
    return std::sin(2 * pi * x / lx) * std::sin(2 * pi * y / ly) * decay;
  }
  Real v() const { return kind == 0 ? 1.0 : 0.0; }
};

Real run(const Case &cs, Int nx) {
  auto mesh = std::make_unique<PlanarHexagonalMesh>(nx, nx, cs.lx / nx, 1);
  ShallowWaterParams params;
  params.m_f0 = 0;
  params.m_disable_h_tendency = true;
  params.m_disable_vn_tendency = true;
  params.m_ntracers = 1;
  if (cs.kind == 1)
    params.m_eddy_diff2 = cs.kappa;
  if (cs.kind == 2)
    params.m_eddy_diff4 = cs.kappa;
  ShallowWaterModel model(mesh.get(), params);
  ShallowWaterState state(mesh.get(), params);
  LSRKStepper stepper(model);
  Real timeend, dt;
  if (cs.kind == 0) {
    timeend = 1;
    dt = 0.5 * mesh->m_dc;
  } else if (cs.kind == 1) {
    timeend = 2;
    dt = mesh->m_dc * mesh->m_dc / (4 * cs.kappa);
  } else {
    timeend = 2;
    dt = std::pow(mesh->m_dc, 4) / (8 * cs.kappa);
  }
  const Int nsteps = Int(std::ceil(timeend / dt));
  dt = timeend / nsteps;
  const Int C = mesh->m_ncells, E = mesh->m_nedges;
  std::vector<Real> h(C), tr(C), exact(C), vn(E);
  for (Int c = 0; c < C; ++c) {
    const Real x = mesh->m_x_cell[c], y = mesh->m_y_cell[c];
    h[c] = cs.h(x, y);
    tr[c] = cs.tr(x, y, 0);
    exact[c] = cs.tr(x, y, timeend);
  }
  for (Int e = 0; e < E; ++e)
    vn[e] = std::cos(mesh->m_angle_edge[e]) * cs.v() +
            std::sin(mesh->m_angle_edge[e]) * cs.v();
  state.upload(h, vn, tr);
  for (Int step = 0; step < nsteps; ++step)
    stepper.do_step(step * dt, dt, state);
  std::vector<Real> hf, vf, tf;
  state.download(hf, vf, tf);
  Real err = 0;
  for (Int c = 0; c < C; ++c)
    err += (exact[c] - tf[c]) * (exact[c] - tf[c]);
  return std::sqrt(err / (mesh->m_nx * mesh->m_ny));
}

int main(int argc, char **argv) {
  const char *which = argc > 1 ? argv[1] : "advection";
  Case cs{};
  Int nx;
  if (!std::strcmp(which, "advection")) {
    cs = {0, 1.0, std::sqrt(3.0) / 2, 0.0};
    nx = 50;
  } else if (!std::strcmp(which, "diffusion")) {
    cs = {1, 10.0, std::sqrt(3.0) / 2 * 10.0, 1.0};
    nx = 16;
  } else if (!std::strcmp(which, "hyperdiffusion")) {
    cs = {2, 10.0, std::sqrt(3.0) / 2 * 10.0, 1.0};
    nx = 16;
  } else {
    std::printf("unknown case %s\n", which);
    return 2;
  }
  const Real e0 = run(cs, nx), e1 = run(cs, 2 * nx);
  const Real rate = std::log2(e0 / e1);
  std::printf("Tracer %s convergence\n0 %.9g\n1 %.9g %.6f\n", which, e0, e1,
              rate);
  if (!(std::abs(rate - 2) < 0.05)) {
    std::printf("FAIL: rate %.4f\n", rate);
    return 1;
  }
  return 0;
}
