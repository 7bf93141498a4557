"""1000-step parity with the oracle on the setups of the reference's
convergence and conservation tests.

Each case but the last takes the mesh, stepper, enabled terms, coefficients
and time step of one reference test (test/double_vortex.cpp, test/tracer_*_convergence.cpp,
test/nonlinear_swe_convergence.cpp) and runs 1000 steps on the GPU and on
the oracle from the same seeded initial state (a stand-in for the test's
analytic one), then compares h, vn and the tracers.  The manufactured
solution's forcing hook is not modelled by the oracle, so that case runs the
same physics unforced.

Bound (normwise relative, max|gpu - oracle| / max|oracle|): <= 1e-10 after
1000 steps.  The kernels regroup the reference's FP64 sums, so the states
agree to accumulated round-off, not bit for bit."""
import math

import numpy as np
import pytest

import omega_playground_gb300 as og
import pyoracle
from helpers import rel_diff
from omega_playground_gb300.workloads import uniform

pytestmark = pytest.mark.gpu

TOL = 1e-10
NSTEPS = 1000


def seeded_state(om, T, seed, h0, hs, vs, uniform_flow=False):
    """Smooth fields with a seeded phase: h = h0 + hs cos(kx x + p) sin(ky y),
    vn = the normal component of the velocity (vs sin(ky y), vs cos(kx x))
    (or of the uniform (vs, vs) when uniform_flow, as in the reference's
    advection test), tr = h times a positive concentration."""
    C_, E, K = om.ncells, om.nedges, om.nlayers
    kx, ky = 2 * math.pi / om.period_x, 2 * math.pi / om.period_y
    ph = 2 * math.pi * float(uniform(seed, 1)[0])
    xc, yc = om.x_cell[:, None], om.y_cell[:, None]
    xe, ye = om.x_edge[:, None], om.y_edge[:, None]
    lev = np.arange(K)[None, :]
    h = h0 + hs * np.cos(kx * xc + ph + 0.3 * lev) * np.sin(ky * yc)
    if uniform_flow:
        ux, uy = vs + 0 * xe, vs + 0 * ye
    else:
        ux, uy = vs * np.sin(ky * ye + ph), vs * np.cos(kx * xe)
    vn = (np.cos(om.angle_edge)[:, None] * ux +
          np.sin(om.angle_edge)[:, None] * uy) * np.ones((1, K))
    tr = np.stack([h * (1.5 + np.sin(kx * (l + 1) * xc) * np.cos(ky * yc))
                   for l in range(T)]) if T else np.zeros((0, C_, K))
    return np.ascontiguousarray(h), np.ascontiguousarray(vn), tr


CASES = {
    # test/double_vortex.cpp: nx = 25, ny = 29 (odd), LSRK5, cfl 0.1,
    # f0 = 6.147e-5, g = 9.80616, no dissipation, h ~ 750 m
    "double_vortex": dict(nx=25, ny=29, dc=5e6 / 25, K=1, T=0, kind="lsrk",
                          f0=0.00006147, grav=9.80616, h0=750.0, hs=75.0,
                          vs=1.0, cfl=0.1),
    # test/tracer_advection_convergence.cpp: frozen h and vn, LSRK5, cfl 0.5
    "tracer_advection": dict(nx=50, ny=50, dc=1.0 / 50, K=1, T=1,
                             kind="lsrk", disable=True, h0=2.0, hs=0.5,
                             vs=1.0, cfl=0.5, uniform_flow=True),
    # test/tracer_diffusion_convergence.cpp: kappa2 = 1, Lx = 10, h = 1,
    # dt = dc^2 / 4
    "tracer_diffusion": dict(nx=16, ny=16, dc=10.0 / 16, K=1, T=1,
                             kind="lsrk", disable=True, eddy_diff2=1.0,
                             h0=1.0, hs=0.0, vs=0.0, dt_pow=2, dt_div=4),
    # test/tracer_hyperdiffusion_convergence.cpp: kappa4 = 1, dt = dc^4 / 8
    "tracer_hyperdiffusion": dict(nx=16, ny=16, dc=10.0 / 16, K=1, T=1,
                                  kind="lsrk", disable=True, eddy_diff4=1.0,
                                  h0=1.0, hs=0.0, vs=0.0, dt_pow=4, dt_div=8),
    # test/nonlinear_swe_convergence.cpp without its forcing: Lx = 1e7 m,
    # h0 = 1000, f0 = 1e-4, g = 9.80616, RK4, dt = 3 s per km of dc, nx = 50
    "nonlinear_swe": dict(nx=50, ny=50, dc=1e7 / 50, K=1, T=0, kind="rk4",
                          f0=1e-4, grav=9.80616, h0=1000.0, hs=1.0, vs=0.1,
                          dt_per_km=3.0),
    # every term on (all four dissipation terms, 2 tracers), RK4, 3 levels,
    # at the 64x64 workload's spacing and a 0.2 gravity-wave CFL
    "rk4_all_terms": dict(nx=12, ny=10, dc=1e4, K=3, T=2, kind="rk4",
                          f0=1e-4, grav=9.81, visc_del2=1e3, visc_del4=1e9,
                          eddy_diff2=1e3, eddy_diff4=1e9, h0=1000.0, hs=5.0,
                          vs=0.1, cfl=0.2),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_1000_steps_against_oracle(name):
    c = CASES[name]
    om = pyoracle.OracleMesh(c["nx"], c["ny"], c["dc"], c["K"])
    disable = c.get("disable", False)
    kw = dict(f0=c.get("f0", 0.0), grav=c.get("grav", 9.81),
              visc_del2=c.get("visc_del2", 0.0),
              visc_del4=c.get("visc_del4", 0.0),
              eddy_diff2=c.get("eddy_diff2", 0.0),
              eddy_diff4=c.get("eddy_diff4", 0.0), ntracers=c["T"],
              disable_h_tendency=disable, disable_vn_tendency=disable)
    omd = pyoracle.OracleModel(om, **kw)
    mesh = og.PlanarHexagonalMesh(c["nx"], c["ny"], c["dc"], c["K"])
    params = og.ShallowWaterParams(
        m_f0=kw["f0"], m_grav=kw["grav"], m_visc_del2=kw["visc_del2"],
        m_visc_del4=kw["visc_del4"], m_eddy_diff2=kw["eddy_diff2"],
        m_eddy_diff4=kw["eddy_diff4"], m_ntracers=c["T"],
        m_disable_h_tendency=disable, m_disable_vn_tendency=disable)
    model = og.ShallowWaterModel(mesh, params)
    x0 = seeded_state(om, c["T"], 4000 + len(name), c["h0"], c["hs"], c["vs"],
                      c.get("uniform_flow", False))
    if "cfl" in c:
        speed = math.sqrt(kw["grav"] * c["h0"]) if not disable else c["vs"]
        dt = c["cfl"] * c["dc"] / max(speed, 1e-30)
    elif "dt_per_km" in c:
        dt = c["dt_per_km"] * c["dc"] / 1e3
    else:
        dt = c["dc"] ** c["dt_pow"] / c["dt_div"]
    nstages = 4 if c["kind"] == "rk4" else 5
    want = omd.step(*(a.copy() for a in x0), 0.0, dt, NSTEPS, kind=c["kind"],
                    nstages=nstages)
    S = og.ShallowWaterState(mesh, params)
    S.upload(*x0)
    st = og.RK4Stepper(model) if c["kind"] == "rk4" else og.LSRKStepper(model, 5)
    st.step(S, 0.0, dt, NSTEPS)
    got = S.download()
    for field, g, w in zip(("h", "vn", "tr"), got, want):
        assert np.all(np.isfinite(w)), field
        assert rel_diff(g, w) <= TOL, (field, rel_diff(g, w))
    # the run did something: the state moved away from the initial one
    moved = max(rel_diff(g, a) for g, a in zip(got, x0) if a.size)
    assert moved > 1e-8, moved
