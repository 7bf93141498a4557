// Manufactured-solution convergence of the full nonlinear model with RK4 on
// the GB300 path (re-hosts test/nonlinear_swe_convergence.cpp: travelling
// wave, forcing through an additional_tendency override, L2 error of h after
// 10 h, nx = 50 and 100, rate 2 +- 0.05).
#include <omega_gpu.hpp>

#include <cstdio>
#include <memory>

using namespace omega;

struct ManufacturedSolution {
  Real m_grav = 9.80616;
  Real m_f0 = 1e-4;
  Real m_lx = 10000 * 1e3;
  Real m_ly = std::sqrt(3.0) / 2 * m_lx;
  Real m_eta0 = 1;
  Real m_h0 = 1000;
  Real m_kx = 2 * (2 * pi / m_lx);
  Real m_ky = 2 * (2 * pi / m_ly);
  Real m_omega = std::sqrt(m_grav * m_h0 * (m_kx * m_kx + m_ky * m_ky));

  __host__ __device__ Real phase(Real x, Real y, Real t) const {
    return m_kx * x + m_ky * y - m_omega * t;
  }
  __host__ __device__ Real h(Real x, Real y, Real t) const {
    return m_h0 + m_eta0 * sin(phase(x, y, t));
  }
  __host__ __device__ Real v(Real x, Real y, Real t) const {
    return m_eta0 * cos(phase(x, y, t)); // vx = vy
  }
  __host__ __device__ Real h_tend(Real x, Real y, Real t) const {
    const Real p = phase(x, y, t);
    return m_eta0 * (-m_h0 * (m_kx + m_ky) * sin(p) - m_omega * cos(p) +
                     m_eta0 * (m_kx + m_ky) * cos(2 * p));
  }
  __host__ __device__ Real vx_tend(Real x, Real y, Real t) const {
    const Real p = phase(x, y, t);
    return m_eta0 * ((-m_f0 + m_grav * m_kx) * cos(p) + m_omega * sin(p) -
                     m_eta0 * (m_kx + m_ky) * sin(2 * p) / 2);
  }
  __host__ __device__ Real vy_tend(Real x, Real y, Real t) const {
    const Real p = phase(x, y, t);
    return m_eta0 * ((m_f0 + m_grav * m_ky) * cos(p) + m_omega * sin(p) -
                     m_eta0 * (m_kx + m_ky) * sin(2 * p) / 2);
  }
};

__global__ void add_forcing(ManufacturedSolution ms, Real2d h_tend,
                            Real2d vn_tend, const Real *xc, const Real *yc,
                            const Real *xe, const Real *ye, const Real *ang,
                            Int ncells, Int nedges, Int K, Real t) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < (long long)ncells * K) {
    const Int c = Int(i / K), k = Int(i % K);
    h_tend(c, k) += ms.h_tend(xc[c], yc[c], t);
  }
  if (i < (long long)nedges * K) {
    const Int e = Int(i / K), k = Int(i % K);
    vn_tend(e, k) += cos(ang[e]) * ms.vx_tend(xe[e], ye[e], t) +
                     sin(ang[e]) * ms.vy_tend(xe[e], ye[e], t);
  }
}

struct ManufacturedShallowWaterModel : ShallowWaterModel {
  ManufacturedSolution m_ms;
  ManufacturedShallowWaterModel(MPASMesh *mesh, const ManufacturedSolution &ms)
      : ShallowWaterModel(mesh, ShallowWaterParams{ms.m_f0, ms.m_grav, 0}),
        m_ms(ms) {}
  void additional_tendency(Real2d h_tend, Real2d vn_tend, RealConst2d,
                           RealConst2d, Real t) const override {
    const MPASMesh *m = m_mesh;
    const long long n = (long long)m->m_nedges * m->m_nlayers;
    add_forcing<<<unsigned((n + 255) / 256), 256>>>(
        m_ms, h_tend, vn_tend, m->d_x_cell.data(), m->d_y_cell.data(),
        m->d_x_edge.data(), m->d_y_edge.data(), m->d_angle_edge.data(),
        m->m_ncells, m->m_nedges, m->m_nlayers, t);
  }
};

Real run(Int n) {
  ManufacturedSolution ms;
  auto mesh = std::make_unique<PlanarHexagonalMesh>(n, n, ms.m_lx / n);
  ManufacturedShallowWaterModel model(mesh.get(), ms);
  ShallowWaterState state(mesh.get(), model.m_params);
  RK4Stepper stepper(model);
  const Real timeend = 10 * 60 * 60;
  Real dt = 3 * mesh->m_dc / 1e3;
  const Int nsteps = Int(std::ceil(timeend / dt));
  dt = timeend / nsteps;
  const Int K = mesh->m_nlayers;
  std::vector<Real> h(size_t(mesh->m_ncells) * K), vn(size_t(mesh->m_nedges) * K),
      hexact(h.size());
  for (Int c = 0; c < mesh->m_ncells; ++c)
    for (Int k = 0; k < K; ++k) {
      h[c * K + k] = ms.h(mesh->m_x_cell[c], mesh->m_y_cell[c], 0);
      hexact[c * K + k] = ms.h(mesh->m_x_cell[c], mesh->m_y_cell[c], timeend);
    }
  for (Int e = 0; e < mesh->m_nedges; ++e)
    for (Int k = 0; k < K; ++k) {
      const Real x = mesh->m_x_edge[e], y = mesh->m_y_edge[e];
      vn[e * K + k] = std::cos(mesh->m_angle_edge[e]) * ms.v(x, y, 0) +
                      std::sin(mesh->m_angle_edge[e]) * ms.v(x, y, 0);
    }
  state.upload(h, vn);
  for (Int step = 0; step < nsteps; ++step)
    stepper.do_step(step * dt, dt, state);
  std::vector<Real> hf, vf, tf;
  state.download(hf, vf, tf);
  Real err = 0;
  for (size_t i = 0; i < hf.size(); ++i)
    err += (hexact[i] - hf[i]) * (hexact[i] - hf[i]);
  return std::sqrt(err / (mesh->m_nx * mesh->m_ny));
}

int main() {
  Real err[2];
  Int nx = 50;
  for (Int l = 0; l < 2; ++l, nx *= 2)
    err[l] = run(nx);
  const Real rate = std::log2(err[0] / err[1]);
  std::printf("Manufactured solution convergence\n0 %.9g\n1 %.9g %.6f\n",
              err[0], err[1], rate);
  if (!(std::abs(rate - 2) < 0.05)) {
    std::printf("FAIL: rate %.4f\n", rate);
    return 1;
  }
  return 0;
}
