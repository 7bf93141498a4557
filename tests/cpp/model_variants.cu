// The C++ drop-in's model variants against twins made through the C ABI:
// LinearShallowWaterModel (shallow_water_hierarchical.cpp:676-775) and the
// opt-in bottom drag (swg_model_options.apply_drag).  Tendencies and three
// RK4 / LSRK5 steps must be bitwise equal.  Also: an exception thrown by an
// additional_tendency override (shallow_water_model.hpp:42-44) reaches the
// caller of compute_tendency / do_steps with its own type, and the model
// works normally afterwards.  Exits non-zero on failure.
#include <omega_gpu.hpp>

#include <cstdint>
#include <cstdio>
#include <vector>

using namespace omega;

namespace {

struct Fields {
  std::vector<Real> h, vn, tr;
  bool operator==(const Fields &o) const {
    return h == o.h && vn == o.vn && tr == o.tr;
  }
};

Fields fields(const ShallowWaterState &s) {
  Fields f;
  s.download(f.h, f.vn, f.tr);
  return f;
}

// tendency and stepped states of a C++ model and of a raw C-ABI twin
bool compare(const char *name, ShallowWaterModel &model, swg_model twin,
             const MPASMesh &mesh, const ShallowWaterParams &p,
             const Fields &x) {
  bool ok = true;
  {
    ShallowWaterState s(&mesh, p), t(&mesh, p), t2(&mesh, p);
    s.upload(x.h, x.vn, x.tr);
    model.compute_tendency(t, s, 0.0);
    swg_check(swg_compute_tendency(twin, t2.handle(), s.handle(), 0.0,
                                   SWG_ADD_REPLACE, nullptr));
    ok = ok && fields(t) == fields(t2);
  }
  for (int kind : {SWG_STEPPER_RK4, SWG_STEPPER_LSRK}) {
    ShallowWaterState a(&mesh, p), b(&mesh, p);
    a.upload(x.h, x.vn, x.tr);
    b.upload(x.h, x.vn, x.tr);
    if (kind == SWG_STEPPER_RK4) {
      RK4Stepper st(model);
      st.do_steps(0, 20, a, 3);
    } else {
      LSRKStepper st(model, 5);
      st.do_steps(0, 20, a, 3);
    }
    swg_stepper raw = nullptr;
    swg_check(swg_stepper_create(twin, kind, 5, &raw));
    swg_check(swg_step(raw, b.handle(), 0, 20, 3, 1, nullptr));
    swg_stepper_destroy(raw);
    ok = ok && fields(a) == fields(b);
  }
  std::printf("%s: bitwise equal to the C ABI twin %d\n", name, ok);
  return ok;
}

Fields state(const MPASMesh &m, int ntr) {
  const size_t C = size_t(m.m_ncells) * m.m_nlayers,
               E = size_t(m.m_nedges) * m.m_nlayers;
  Fields f;
  uint64_t z = 777;
  auto next = [&z]() {
    z = z * 6364136223846793005ull + 1442695040888963407ull;
    return double(z >> 11) * 0x1.0p-53;
  };
  for (size_t i = 0; i < C; ++i) f.h.push_back(1000 + 3 * next());
  for (size_t i = 0; i < E; ++i) f.vn.push_back(0.2 * (next() - 0.5));
  for (size_t i = 0; i < ntr * C; ++i) f.tr.push_back(f.h[i % C] * next());
  return f;
}

struct HookError {
  int calls;
};

// a forcing override that throws while armed
struct ThrowingModel : ShallowWaterModel {
  using ShallowWaterModel::ShallowWaterModel;
  mutable int calls = 0;
  bool arm = true;
  void additional_tendency(Real2d, Real2d, RealConst2d, RealConst2d,
                           Real) const override {
    ++calls;
    if (arm)
      throw HookError{calls};
  }
};

bool hook_exceptions(MPASMesh &mesh) {
  ShallowWaterParams p;
  p.m_f0 = 1e-4;
  p.m_visc_del2 = 1e3;
  p.m_ntracers = 1;
  const Fields x = state(mesh, 1);
  ThrowingModel model(&mesh, p);
  ShallowWaterState s(&mesh, p), t(&mesh, p);
  s.upload(x.h, x.vn, x.tr);
  int rethrown = 0;
  try {
    model.compute_tendency(t, s, 0.0);
  } catch (const HookError &e) {
    rethrown += e.calls == 1;
  }
  RK4Stepper st(model);
  try { // the first hook call throws; the rest of the call skips the hook
    st.do_steps(0, 20, s, 2);
  } catch (const HookError &e) {
    rethrown += e.calls == 2 && model.calls == 2;
  }
  // disarmed: the same results as a model that never threw
  model.arm = false;
  ThrowingModel fresh(&mesh, p);
  fresh.arm = false;
  RK4Stepper st2(fresh);
  ShallowWaterState a(&mesh, p), b(&mesh, p), ta(&mesh, p), tb(&mesh, p);
  a.upload(x.h, x.vn, x.tr);
  b.upload(x.h, x.vn, x.tr);
  model.compute_tendency(ta, a, 0.0);
  fresh.compute_tendency(tb, b, 0.0);
  bool same = fields(ta) == fields(tb);
  st.do_steps(0, 20, a, 2);
  st2.do_steps(0, 20, b, 2);
  same = same && fields(a) == fields(b);
  std::printf("hook exceptions: rethrown %d, usable after %d\n",
              rethrown == 2, same);
  return rethrown == 2 && same;
}

} // namespace

int main() {
  PlanarHexagonalMesh mesh(10, 8, 1e4, 3);
  bool ok = true;
  {
    LinearShallowWaterParams lp;
    lp.m_f0 = 1e-4;
    lp.m_h0 = 850;
    LinearShallowWaterModel lin(&mesh, lp);
    swg_params raw{lp.m_f0, lp.m_grav, 0, 0, 0, 0, 0, 0, 0, 0};
    swg_model twin = nullptr;
    swg_check(swg_linear_model_create(mesh.m_handle, &raw, 850.0, &twin));
    ok = compare("LinearShallowWaterModel", lin, twin, mesh, lp,
                 state(mesh, 0)) && ok;
    swg_model_destroy(twin);
  }
  {
    ShallowWaterParams p;
    p.m_f0 = 1e-4;
    p.m_visc_del2 = 1e3;
    p.m_drag_coeff = 2e-3;
    p.m_ntracers = 1;
    ShallowWaterModel drag(&mesh, p, swg_model_options{0, 0, 1});
    swg_params raw{p.m_f0, p.m_grav, p.m_drag_coeff, p.m_visc_del2, 0, 0, 0,
                   1, 0, 0};
    swg_model_options o{0, 0, 1};
    swg_model twin = nullptr;
    swg_check(swg_model_create_ex(mesh.m_handle, &raw, &o, &twin));
    ok = compare("bottom drag", drag, twin, mesh, p, state(mesh, 1)) && ok;
    swg_model_destroy(twin);
  }
  ok = hook_exceptions(mesh) && ok;
  std::printf("%s\n", ok ? "PASS" : "FAIL");
  return ok ? 0 : 1;
}
