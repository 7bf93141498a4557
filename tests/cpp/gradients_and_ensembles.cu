// The C++ drop-in's ensemble and gradient classes, used the way a reference
// user would: (1) a dot-product test of the checkpointed adjoint against the
// tangent-linear model over 10 RK4 steps with every term on,
// <J dx0, lamN> = <dx0, J^T lamN> to 1e-12; (2) three members of different
// sizes advanced by EnsembleStepper, and by HostStepper from host arrays,
// equal, bit for bit, the same members advanced one at a time by
// RK4Stepper; (3) three members' gradients through
// CheckpointedAdjointEnsemble (two share a schedule and run in lockstep)
// equal, bit for bit, each member's own CheckpointedAdjoint.  Exits
// non-zero on failure.
#include <omega_gpu.hpp>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <memory>
#include <vector>

using namespace omega;

namespace {

struct SplitMix {
  uint64_t s;
  double next() { // uniform in [0, 1)
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return double(z >> 11) * 0x1.0p-53;
  }
};

struct Fields {
  std::vector<Real> h, vn, tr;
};

Fields random_state(const MPASMesh &m, Int ntr, uint64_t seed, Real h0,
                    Real hs, Real vs, Real ts) {
  SplitMix r{seed};
  const size_t C = size_t(m.m_ncells) * m.m_nlayers;
  const size_t E = size_t(m.m_nedges) * m.m_nlayers;
  Fields f;
  for (size_t i = 0; i < C; ++i)
    f.h.push_back(h0 + hs * (r.next() - 0.5));
  for (size_t i = 0; i < E; ++i)
    f.vn.push_back(vs * (r.next() - 0.5));
  for (Int l = 0; l < ntr; ++l)
    for (size_t i = 0; i < C; ++i)
      f.tr.push_back(ts * (h0 > 0 ? f.h[i] * r.next() : r.next() - 0.5));
  return f;
}

double dot(const Fields &a, const Fields &b) {
  double s = 0;
  for (size_t i = 0; i < a.h.size(); ++i)
    s += a.h[i] * b.h[i];
  for (size_t i = 0; i < a.vn.size(); ++i)
    s += a.vn[i] * b.vn[i];
  for (size_t i = 0; i < a.tr.size(); ++i)
    s += a.tr[i] * b.tr[i];
  return s;
}

Fields download(const ShallowWaterState &s) {
  Fields f;
  s.download(f.h, f.vn, f.tr);
  return f;
}

bool dot_product_test() {
  PlanarHexagonalMesh mesh(12, 10, 1e4, 5);
  ShallowWaterParams p;
  p.m_f0 = 1e-4;
  p.m_visc_del2 = 1e3;
  p.m_visc_del4 = 1e9;
  p.m_eddy_diff2 = 1e3;
  p.m_eddy_diff4 = 1e9;
  p.m_ntracers = 2;
  ShallowWaterModel model(&mesh, p);
  const Real dt = 20, t0 = 0;
  const Int nsteps = 10;
  CheckpointedAdjoint adj(model, 4);

  const Fields x0 = random_state(mesh, 2, 11, 1000, 2, 0.2, 1);
  const Fields dx0 = random_state(mesh, 2, 22, 0, 1, 0.01, 10);
  const Fields lamN = random_state(mesh, 2, 33, 0, 1, 1, 1);
  ShallowWaterState X0(&mesh, p), XN(&mesh, p), DX(&mesh, p), LAM(&mesh, p);
  X0.upload(x0.h, x0.vn, x0.tr);
  DX.upload(dx0.h, dx0.vn, dx0.tr);
  LAM.upload(lamN.h, lamN.vn, lamN.tr);
  adj.forward(X0, t0, dt, nsteps, XN);
  adj.backward(LAM);
  adj.tlm_apply(X0, DX, t0, dt, nsteps);
  const double lhs = dot(download(DX), lamN);
  const double rhs = dot(dx0, download(LAM));
  const double rel = std::fabs(lhs - rhs) / std::fmax(std::fabs(lhs), std::fabs(rhs));
  std::printf("dot_product lhs=%.17e rhs=%.17e rel=%.3e plain_steps=%lld "
              "taped_advances=%lld\n",
              lhs, rhs, rel, adj.plain_steps(), adj.taped_advances());
  return rel <= 1e-12;
}

bool ensemble_test() {
  struct Member {
    std::unique_ptr<PlanarHexagonalMesh> mesh;
    ShallowWaterParams p;
    std::unique_ptr<ShallowWaterModel> model;
    Fields x0;
  };
  const Int nx[3] = {8, 12, 16}, K[3] = {3, 7, 5}, T[3] = {1, 0, 3};
  std::vector<Member> mem(3);
  for (int m = 0; m < 3; ++m) {
    mem[m].mesh = std::make_unique<PlanarHexagonalMesh>(nx[m], nx[m], 1e4, K[m]);
    mem[m].p.m_f0 = 1e-4;
    mem[m].p.m_visc_del2 = 1e3;
    mem[m].p.m_ntracers = T[m];
    mem[m].model = std::make_unique<ShallowWaterModel>(mem[m].mesh.get(), mem[m].p);
    mem[m].x0 = random_state(*mem[m].mesh, T[m], 100 + m, 1000, 2, 0.2, 1);
  }
  const Real dt = 20;
  // one at a time
  std::vector<Fields> ref;
  for (auto &m : mem) {
    ShallowWaterState s(m.mesh.get(), m.p);
    s.upload(m.x0.h, m.x0.vn, m.x0.tr);
    RK4Stepper st(*m.model);
    st.do_steps(0, dt, s, 3);
    ref.push_back(download(s));
  }
  // together
  std::vector<std::unique_ptr<ShallowWaterState>> states;
  std::vector<ShallowWaterModel *> models;
  std::vector<const ShallowWaterState *> sp;
  for (auto &m : mem) {
    states.push_back(std::make_unique<ShallowWaterState>(m.mesh.get(), m.p));
    models.push_back(m.model.get());
    sp.push_back(states.back().get());
  }
  EnsembleStepper ens(models, sp);
  ens.autotune(dt, 1);
  for (int m = 0; m < 3; ++m)
    states[m]->upload(mem[m].x0.h, mem[m].x0.vn, mem[m].x0.tr);
  ens.do_steps(0, dt, 3);
  double worst = 0;
  for (int m = 0; m < 3; ++m) {
    const Fields got = download(*states[m]);
    for (size_t i = 0; i < got.h.size(); ++i)
      worst = std::fmax(worst, std::fabs(got.h[i] - ref[m].h[i]));
    for (size_t i = 0; i < got.vn.size(); ++i)
      worst = std::fmax(worst, std::fabs(got.vn[i] - ref[m].vn[i]));
    for (size_t i = 0; i < got.tr.size(); ++i)
      worst = std::fmax(worst, std::fabs(got.tr[i] - ref[m].tr[i]));
  }
  std::printf("ensemble max_abs_diff=%.3e\n", worst);
  // the same members kept in host arrays, stepped in chunks of 2 levels
  double worst_host = 0;
  for (int m = 0; m < 3; ++m) {
    Fields x = mem[m].x0;
    HostStepper hs(*mem[m].model, true, 4, 2);
    hs.do_steps(0, dt, x.h.data(), x.vn.data(),
                x.tr.empty() ? nullptr : x.tr.data(), 3);
    for (size_t i = 0; i < x.h.size(); ++i)
      worst_host = std::fmax(worst_host, std::fabs(x.h[i] - ref[m].h[i]));
    for (size_t i = 0; i < x.vn.size(); ++i)
      worst_host = std::fmax(worst_host, std::fabs(x.vn[i] - ref[m].vn[i]));
    for (size_t i = 0; i < x.tr.size(); ++i)
      worst_host = std::fmax(worst_host, std::fabs(x.tr[i] - ref[m].tr[i]));
  }
  std::printf("host max_abs_diff=%.3e\n", worst_host);
  return worst == 0.0 && worst_host == 0.0;
}

bool same(const Fields &a, const Fields &b) {
  return a.h == b.h && a.vn == b.vn && a.tr == b.tr;
}

bool adjoint_ensemble_test() {
  struct Member {
    std::unique_ptr<PlanarHexagonalMesh> mesh;
    ShallowWaterParams p;
    std::unique_ptr<ShallowWaterModel> model;
    std::unique_ptr<CheckpointedAdjoint> adj;
    std::unique_ptr<ShallowWaterState> x0, xN, lam;
    Fields f0, g;
  };
  // members 0 and 1: same schedule (4 snapshots, RK4, 2 tracers), different
  // sizes; member 2: 3 snapshots, its own group
  const Int nx[3] = {10, 14, 8}, K[3] = {4, 3, 6}, nsnap[3] = {4, 4, 3};
  const Real dt = 20, t0 = 0;
  const Int nsteps = 9;
  std::vector<Member> mem(3);
  for (int m = 0; m < 3; ++m) {
    Member &u = mem[m];
    u.mesh = std::make_unique<PlanarHexagonalMesh>(nx[m], nx[m] - 2, 1e4, K[m]);
    u.p.m_f0 = 1e-4;
    u.p.m_visc_del2 = 1e3;
    u.p.m_visc_del4 = 1e9;
    u.p.m_eddy_diff2 = 1e3;
    u.p.m_ntracers = 2;
    u.model = std::make_unique<ShallowWaterModel>(u.mesh.get(), u.p);
    u.adj = std::make_unique<CheckpointedAdjoint>(*u.model, nsnap[m]);
    u.x0 = std::make_unique<ShallowWaterState>(u.mesh.get(), u.p);
    u.xN = std::make_unique<ShallowWaterState>(u.mesh.get(), u.p);
    u.lam = std::make_unique<ShallowWaterState>(u.mesh.get(), u.p);
    u.f0 = random_state(*u.mesh, 2, 100 + m, 1000, 2, 0.2, 1);
    u.g = random_state(*u.mesh, 2, 200 + m, 0, 1, 1, 1);
    u.x0->upload(u.f0.h, u.f0.vn, u.f0.tr);
  }
  // each member's own adjoint
  std::vector<Fields> ref(3), refN(3);
  for (Member &u : mem) {
    u.adj->forward(*u.x0, t0, dt, nsteps, *u.xN);
    u.lam->upload(u.g.h, u.g.vn, u.g.tr);
    u.adj->backward(*u.lam);
  }
  for (int m = 0; m < 3; ++m) {
    ref[m] = download(*mem[m].lam);
    refN[m] = download(*mem[m].xN);
  }
  // the same through the ensemble
  std::vector<CheckpointedAdjoint *> adjs;
  std::vector<const ShallowWaterState *> x0s, xNs, lams;
  for (Member &u : mem) {
    adjs.push_back(u.adj.get());
    x0s.push_back(u.x0.get());
    xNs.push_back(u.xN.get());
    lams.push_back(u.lam.get());
  }
  CheckpointedAdjointEnsemble ens(adjs);
  std::vector<int> group_of;
  const Int ngroups = ens.groups(&group_of);
  ens.forward(x0s, t0, dt, nsteps, xNs);
  for (Member &u : mem)
    u.lam->upload(u.g.h, u.g.vn, u.g.tr);
  ens.backward(lams);
  bool ok = ngroups == 2 && group_of[0] == group_of[1] &&
            group_of[0] != group_of[2];
  for (int m = 0; m < 3; ++m)
    ok = ok && same(download(*mem[m].lam), ref[m]) &&
         same(download(*mem[m].xN), refN[m]);
  std::printf("adjoint ensemble groups=%lld bitwise=%d\n", (long long)ngroups,
              ok);
  return ok;
}

} // namespace

int main() {
  const bool a = dot_product_test();
  const bool b = ensemble_test();
  const bool c = adjoint_ensemble_test();
  std::printf("%s\n", a && b && c ? "PASS" : "FAIL");
  return a && b && c ? 0 : 1;
}
