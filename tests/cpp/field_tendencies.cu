// The C++ drop-in's auxiliary state and per-field tendency methods
// (shallow_water_model.hpp:18,36-41), used the way a reference user would:
//   model.m_aux_state.compute(h, vn, tr, model.m_f_vertex, &mesh);
//   model.compute_h_tendency(tend.m_h_cell, h, vn, AddMode::replace);
// (1) after compute_tendency(state), the three per-field methods with the
// state's own views reproduce its tendency bit for bit; (2) increment mode
// adds the same values again; (3) m_aux_state.compute of a second state
// changes the views' contents (the mean thickness equals (h0 + h1) / 2 of
// that state's cells); (4) a plain model drops its construction-time hook
// when a stepper is built, without running a tendency, so its first step
// already replays the fused step graph.  Exits non-zero on failure.
#include <omega_gpu.hpp>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>

using namespace omega;

namespace {

struct Fields {
  std::vector<Real> h, vn, tr;
};

Fields random_fields(const MPASMesh &mesh, Int K, Int T, uint64_t seed) {
  const size_t C = size_t(mesh.m_ncells) * K, E = size_t(mesh.m_nedges) * K;
  Fields f;
  f.h.resize(C);
  f.vn.resize(E);
  f.tr.resize(T * C);
  uint64_t z = seed;
  auto next = [&z]() {
    z = z * 6364136223846793005ull + 1442695040888963407ull;
    return double(z >> 11) * 0x1.0p-53;
  };
  for (auto &x : f.h) x = 1000 + 3 * next();
  for (auto &x : f.vn) x = 0.2 * (next() - 0.5);
  for (size_t i = 0; i < f.tr.size(); ++i) f.tr[i] = f.h[i % C] * (0.5 + next());
  return f;
}

Fields download(const ShallowWaterState &s) {
  Fields f;
  s.download(f.h, f.vn, f.tr);
  return f;
}

bool same(const std::vector<Real> &a, const std::vector<Real> &b) {
  if (a.size() != b.size())
    return false;
  for (size_t i = 0; i < a.size(); ++i)
    if (a[i] != b[i])
      return false;
  return true;
}

std::vector<Real> host(RealConst2d v) {
  std::vector<Real> out(v.size());
  if (cudaMemcpy(out.data(), v.data(), out.size() * sizeof(Real),
                 cudaMemcpyDeviceToHost) != cudaSuccess)
    throw std::runtime_error("cudaMemcpy");
  return out;
}

} // namespace

int main() {
  const Int K = 4, T = 2;
  PlanarHexagonalMesh mesh(10, 8, 1e4, K);
  ShallowWaterParams p;
  p.m_f0 = 1e-4;
  p.m_visc_del2 = 1e3;
  p.m_visc_del4 = 1e9;
  p.m_eddy_diff2 = 1e3;
  p.m_eddy_diff4 = 1e9;
  p.m_ntracers = T;
  ShallowWaterModel model(&mesh, p);
  ShallowWaterState a(&mesh, p), b(&mesh, p), full(&mesh, p), part(&mesh, p);
  const Fields fa = random_fields(mesh, K, T, 12345);
  const Fields fb = random_fields(mesh, K, T, 777);
  a.upload(fa.h, fa.vn, fa.tr);
  b.upload(fb.h, fb.vn, fb.tr);
  bool ok = true;

  // (4) the hook of a plain model is dropped when the stepper is built, so
  // the first step already replays the fused step graph: it launches as
  // many kernels as the second (a hooked first step runs the unfused
  // sequence, with more launches)
  {
    ShallowWaterModel fresh(&mesh, p);
    ShallowWaterState s(&mesh, p);
    s.upload(fa.h, fa.vn, fa.tr);
    RK4Stepper stepper(fresh);
    long long n[3] = {swg_kernel_launches(), 0, 0};
    stepper.do_step(0.0, 10.0, s);
    n[1] = swg_kernel_launches();
    stepper.do_step(10.0, 10.0, s);
    n[2] = swg_kernel_launches();
    fence();
    std::printf("kernels of the first and second step: %lld %lld\n",
                n[1] - n[0], n[2] - n[1]);
    ok = ok && n[1] - n[0] == n[2] - n[1];
  }

  // (1) per-field methods after compute_tendency equal it bit for bit
  model.compute_tendency(full, a, 0.0);
  model.compute_h_tendency(part.m_h_cell, a.m_h_cell, a.m_vn_edge,
                           AddMode::replace);
  model.compute_vn_tendency(part.m_vn_edge, a.m_h_cell, a.m_vn_edge,
                            AddMode::replace);
  model.compute_tr_tendency(part.m_tr_cell, a.m_tr_cell, a.m_vn_edge,
                            AddMode::replace);
  const Fields ff = download(full), fp = download(part);
  const bool bitwise = same(ff.h, fp.h) && same(ff.vn, fp.vn) &&
                       same(ff.tr, fp.tr);
  std::printf("per-field methods equal compute_tendency bit for bit %d\n",
              bitwise);
  ok = ok && bitwise;

  // (2) increment adds the same values again
  model.compute_h_tendency(part.m_h_cell, a.m_h_cell, a.m_vn_edge,
                           AddMode::increment);
  model.compute_vn_tendency(part.m_vn_edge, a.m_h_cell, a.m_vn_edge,
                            AddMode::increment);
  model.compute_tr_tendency(part.m_tr_cell, a.m_tr_cell, a.m_vn_edge,
                            AddMode::increment);
  const Fields f2 = download(part);
  bool twice = true;
  for (size_t i = 0; i < ff.h.size(); ++i)
    twice = twice && f2.h[i] == ff.h[i] + ff.h[i];
  for (size_t i = 0; i < ff.vn.size(); ++i)
    twice = twice && f2.vn[i] == ff.vn[i] + ff.vn[i];
  for (size_t i = 0; i < ff.tr.size(); ++i)
    twice = twice && f2.tr[i] == ff.tr[i] + ff.tr[i];
  std::printf("increment adds the tendency again %d\n", twice);
  ok = ok && twice;

  // (3) m_aux_state.compute of state b: its mean thickness
  model.m_aux_state.compute(b.m_h_cell, b.m_vn_edge, b.m_tr_cell,
                            model.m_f_vertex, &mesh);
  fence();
  const std::vector<Real> mh =
      host(model.m_aux_state.m_thickness_aux.m_mean_h_edge);
  double err = 0;
  for (Int e = 0; e < mesh.m_nedges; ++e)
    for (Int k = 0; k < K; ++k) {
      const Int c0 = mesh.m_cells_on_edge[2 * e],
                c1 = mesh.m_cells_on_edge[2 * e + 1];
      const Real ref = 0.5 * (fb.h[size_t(c0) * K + k] + fb.h[size_t(c1) * K + k]);
      err = std::fmax(err, std::fabs(mh[size_t(e) * K + k] - ref));
    }
  const bool aux_ok = err == 0 &&
                      model.m_aux_state.m_thickness_aux.m_flux_h_edge.data() ==
                          model.m_aux_state.m_thickness_aux.m_mean_h_edge.data() &&
                      model.m_aux_state.m_tracer_aux.m_norm_tr_cell.extent(0) == T;
  std::printf("m_aux_state.compute: mean thickness of the new state, max "
              "error %.3e; views bound %d\n", err, aux_ok);
  ok = ok && aux_ok;
  std::printf("%s\n", ok ? "PASS" : "FAIL");
  return ok ? 0 : 1;
}
