// The C++ drop-in's tendency-term members (shallow_water_model.hpp:19-29)
// and m_f_vertex (:32), used the way a reference user would:
//   model.m_pv_flux_edge.m_enabled = false;
//   model.m_f_vertex(iv) = f0 + beta * y   (inside a user kernel)
// (1) every member switched off alone changes exactly the fields its term
// writes (h: thickness advection; vn: PV flux, KE and SSH gradients, del2,
// del4; tracers: advection, del2, del4), reads back false, and gives the
// same tendency, bit for bit, as the same term switched through the C ABI
// on a second model; switching it back restores the all-on tendency;
// (2) a beta plane written through m_f_vertex changes vn's tendency only.
// Exits non-zero on failure.
#include <omega_gpu.hpp>

#include <cstdint>
#include <cstdio>
#include <vector>

using namespace omega;

namespace {

struct Fields {
  std::vector<Real> h, vn, tr;
};

Fields tendency(ShallowWaterModel &model, const ShallowWaterState &s,
                const MPASMesh *mesh, const ShallowWaterParams &p) {
  ShallowWaterState t(mesh, p);
  model.compute_tendency(t, s, 0.0);
  Fields f;
  t.download(f.h, f.vn, f.tr);
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

__global__ void beta_plane(Real1d f, RealConst1d y, Real f0, Real beta,
                           Real y0) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < f.extent(0))
    f(i) = f0 + beta * (y(i) - y0);
}

} // namespace

int main() {
  PlanarHexagonalMesh mesh(10, 8, 1e4, 4);
  ShallowWaterParams p;
  p.m_f0 = 1e-4;
  p.m_visc_del2 = 1e3;
  p.m_visc_del4 = 1e9;
  p.m_eddy_diff2 = 1e3;
  p.m_eddy_diff4 = 1e9;
  p.m_ntracers = 2;
  ShallowWaterModel model(&mesh, p), twin(&mesh, p);
  ShallowWaterState s(&mesh, p);
  {
    const size_t C = size_t(mesh.m_ncells) * 4, E = size_t(mesh.m_nedges) * 4;
    std::vector<Real> h(C), vn(E), tr(2 * C);
    uint64_t z = 12345;
    auto next = [&z]() {
      z = z * 6364136223846793005ull + 1442695040888963407ull;
      return double(z >> 11) * 0x1.0p-53;
    };
    for (auto &x : h) x = 1000 + 3 * next();
    for (auto &x : vn) x = 0.2 * (next() - 0.5);
    for (size_t i = 0; i < 2 * C; ++i) tr[i] = h[i % C] * (0.5 + next());
    s.upload(h, vn, tr);
  }
  const Fields all = tendency(model, s, &mesh, p);
  struct Case {
    TendencyTerm *term;
    int id;
    const char *name;
    bool h, vn, tr; // fields the term writes
  } cases[] = {
      {&model.m_thickness_hadv_cell, SWG_TERM_THICKNESS_HADV, "thickness_hadv", 1, 0, 0},
      {&model.m_pv_flux_edge, SWG_TERM_PV_FLUX, "pv_flux", 0, 1, 0},
      {&model.m_ke_grad_edge, SWG_TERM_KE_GRAD, "ke_grad", 0, 1, 0},
      {&model.m_ssh_grad_edge, SWG_TERM_SSH_GRAD, "ssh_grad", 0, 1, 0},
      {&model.m_vel_diff_edge, SWG_TERM_VEL_DIFF, "vel_diff", 0, 1, 0},
      {&model.m_vel_hyperdiff_edge, SWG_TERM_VEL_HYPERDIFF, "vel_hyperdiff", 0, 1, 0},
      {&model.m_tracer_hadv_cell, SWG_TERM_TRACER_HADV, "tracer_hadv", 0, 0, 1},
      {&model.m_tracer_diff_cell, SWG_TERM_TRACER_DIFF, "tracer_diff", 0, 0, 1},
      {&model.m_tracer_hyperdiff_cell, SWG_TERM_TRACER_HYPERDIFF, "tracer_hyperdiff", 0, 0, 1},
  };
  bool ok = true;
  for (const Case &c : cases) {
    c.term->m_enabled = false;
    const bool reads_off = !bool(c.term->m_enabled);
    const Fields off = tendency(model, s, &mesh, p);
    swg_check(swg_model_set_term_enabled(twin.m_handle, c.id, 0));
    const Fields ref = tendency(twin, s, &mesh, p);
    swg_check(swg_model_set_term_enabled(twin.m_handle, c.id, 1));
    c.term->m_enabled = true;
    const Fields back = tendency(model, s, &mesh, p);
    const bool fields_ok = same(off.h, all.h) != c.h &&
                           same(off.vn, all.vn) != c.vn &&
                           same(off.tr, all.tr) != c.tr;
    const bool twin_ok = same(off.h, ref.h) && same(off.vn, ref.vn) &&
                         same(off.tr, ref.tr);
    const bool back_ok = same(back.h, all.h) && same(back.vn, all.vn) &&
                         same(back.tr, all.tr) && bool(c.term->m_enabled);
    std::printf("%-17s off reads false %d, changes only its fields %d, "
                "equals the C ABI switch %d, restored %d\n",
                c.name, reads_off, fields_ok, twin_ok, back_ok);
    ok = ok && reads_off && fields_ok && twin_ok && back_ok;
  }
  // a beta plane through m_f_vertex
  DeviceArray<Real> yv(mesh.m_y_vertex);
  beta_plane<<<(mesh.m_nvertices + 127) / 128, 128>>>(
      model.m_f_vertex, yv.view(), 1e-4, 1.6e-11, 0.5 * mesh.m_period_y);
  swg_check(cudaGetLastError() == cudaSuccess ? SWG_OK : SWG_ERR_CUDA);
  fence();
  const Fields beta = tendency(model, s, &mesh, p);
  const bool beta_ok = same(beta.h, all.h) && !same(beta.vn, all.vn) &&
                       same(beta.tr, all.tr);
  std::printf("beta plane through m_f_vertex changes only vn %d\n", beta_ok);
  ok = ok && beta_ok;
  std::printf("%s\n", ok ? "PASS" : "FAIL");
  return ok ? 0 : 1;
}
