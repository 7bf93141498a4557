"""GPU path against the reference: golden fixtures and the oracle.

Bounds (normwise relative, max|gpu - ref| / max|ref|, written per test):
  tendencies and auxiliary fields of one evaluation   <= 1e-12
  state after N steps (N <= 10)                       <= 1e-12
  state after 1000 steps (lsrk5_1000_steps fixture)   <= 1e-10
The kernels regroup the reference's FP64 sums (hoisted coefficients, fused
multiply-adds, Newton reciprocals), so agreement is to round-off, not bit
for bit."""
import numpy as np
import pytest

import omega_playground_gb300 as og
from helpers import STEPPER_KIND, golden_names, load_golden, oracle_model, rel_diff
from omega_playground_gb300.workloads import WORKLOADS, initial_state

pytestmark = pytest.mark.gpu

TOL = 1e-12


def gpu_setup(cfg):
    mesh = og.PlanarHexagonalMesh(cfg["nx"], cfg["ny"], cfg["dc"], cfg["K"])
    params = og.ShallowWaterParams(
        m_f0=cfg["f0"], m_grav=cfg["grav"], m_visc_del2=cfg["visc_del2"],
        m_visc_del4=cfg["visc_del4"], m_eddy_diff2=cfg["eddy_diff2"],
        m_eddy_diff4=cfg["eddy_diff4"], m_ntracers=cfg["T"],
        m_disable_h_tendency=cfg["disable_h"],
        m_disable_vn_tendency=cfg["disable_vn"])
    model = og.ShallowWaterModel(mesh, params)
    return mesh, params, model


def make_stepper(model, stepper_code):
    kind, ns = STEPPER_KIND[stepper_code]
    return og.RK4Stepper(model) if kind == "rk4" else og.LSRKStepper(model, ns)


@pytest.mark.parametrize("name", golden_names())
def test_golden_tendency(name):
    g = load_golden(name)
    cfg = g["cfg"]
    mesh, params, model = gpu_setup(cfg)
    state = og.ShallowWaterState(mesh, params)
    state.upload(g["in_h"], g["in_vn"], g["in_tr"])
    tend = og.ShallowWaterState(mesh, params)
    model.compute_tendency(tend, state, 0.0)
    th, tv, tt = tend.download()
    assert rel_diff(th, g["tend_h"]) <= TOL
    assert rel_diff(tv, g["tend_vn"]) <= TOL
    assert rel_diff(tt, g["tend_tr"]) <= TOL


@pytest.mark.parametrize("name", golden_names())
def test_golden_aux_fields(name):
    """Every intermediate the kernels keep, against the reference's own
    auxiliary arrays (same quantities, regrouped where noted)."""
    g = load_golden(name)
    cfg = g["cfg"]
    mesh, params, model = gpu_setup(cfg)
    state = og.ShallowWaterState(mesh, params)
    state.upload(g["in_h"], g["in_vn"], g["in_tr"])
    tend = og.ShallowWaterState(mesh, params)
    model.compute_tendency(tend, state, 0.0)
    K = cfg["K"]
    checks = {"thick_flux_edge": g["mean_h_edge"] * g["in_vn"]}
    if not cfg["disable_vn"]:
        checks["q_vertex"] = g["norm_rvort_vertex"] + g["norm_pvort_vertex"]
        checks["pv_edge"] = 2 * (g["norm_rvort_edge"] + g["norm_pvort_edge"])
        checks["ke_cell"] = g["ke_cell"]
        if cfg["visc_del2"] > 0 or cfg["visc_del4"] > 0:
            checks["rvort_vertex"] = g["rvort_vertex"]
            checks["vel_div_cell"] = g["vel_div_cell"]
        if cfg["visc_del4"] > 0:
            checks["vel_del2_edge"] = g["vel_del2_edge"]
            checks["vel_del2_rvort_vertex"] = g["vel_del2_rvort_vertex"]
            checks["vel_del2_div_cell"] = g["vel_del2_div_cell"]
    if cfg["T"] > 0:
        checks["norm_tr_cell"] = g["norm_tr_cell"]
        if cfg["eddy_diff4"] > 0:
            checks["tracer_del2_cell"] = g["tracer_del2_cell"]
        if cfg["eddy_diff2"] > 0 or cfg["eddy_diff4"] > 0:
            checks["mean_h_edge"] = g["mean_h_edge"]
    for name_, ref in checks.items():
        got = model.aux(name_)
        assert got.size == ref.size, name_
        assert rel_diff(got, ref.ravel()) <= TOL, name_
    assert K >= 1


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("use_graph", [False, True])
def test_golden_steps(name, use_graph):
    g = load_golden(name)
    cfg = g["cfg"]
    if cfg["stepper"] not in STEPPER_KIND:
        pytest.skip("no stepper")
    mesh, params, model = gpu_setup(cfg)
    state = og.ShallowWaterState(mesh, params)
    state.upload(g["in_h"], g["in_vn"], g["in_tr"])
    stepper = make_stepper(model, cfg["stepper"])
    stepper.step(state, cfg["t0"], cfg["dt"], cfg["nsteps"], use_graph=use_graph)
    h, vn, tr = state.download()
    # round-off accumulates: 1e-12 up to 10 steps, 1e-10 for the 1000-step run
    tol = TOL if cfg["nsteps"] <= 10 else 1e-10
    assert rel_diff(h, g["h_final"]) <= tol
    assert rel_diff(vn, g["vn_final"]) <= tol
    assert rel_diff(tr, g["tr_final"]) <= tol
    assert abs(og.mass_integral(state, model) - g["mass1"][0]) <= \
        1e-13 * abs(g["mass1"][0])


def _oracle_vs_gpu(wl, nsteps, use_graph=True):
    cfg = dict(nx=wl.nx, ny=wl.ny, dc=wl.dc, K=wl.nlayers, T=wl.ntracers,
               f0=wl.f0, grav=wl.grav, visc_del2=wl.visc_del2,
               visc_del4=wl.visc_del4, eddy_diff2=wl.eddy_diff2,
               eddy_diff4=wl.eddy_diff4, disable_h=False, disable_vn=False)
    mesh, params, model = gpu_setup(cfg)
    h0, vn0, tr0 = initial_state(mesh, wl)
    state = og.ShallowWaterState(mesh, params)
    state.upload(h0, vn0, tr0)
    stepper = og.RK4Stepper(model) if wl.stepper == "rk4" else \
        og.LSRKStepper(model, wl.nstages)
    stepper.step(state, 0.0, wl.dt, nsteps, use_graph=use_graph)
    got = state.download()
    _, omd = oracle_model(cfg)
    ref = [np.ascontiguousarray(x) for x in (h0, vn0, tr0)]
    omd.step(*ref, 0.0, wl.dt, nsteps, wl.stepper, wl.nstages)
    return got, ref


def test_rk4_64x64_workload_10_steps():
    """The 64x64x64, 1-tracer RK4 workload, 10 steps, against the oracle."""
    wl = WORKLOADS["rk4_64x64"]
    (h, vn, tr), (rh, rvn, rtr) = _oracle_vs_gpu(wl, 10)
    assert rel_diff(h, rh) <= TOL
    assert rel_diff(vn, rvn) <= TOL
    assert rel_diff(tr, rtr) <= TOL


def test_lsrk5_all_terms_reduced_10_steps():
    """The 512x512 workload's physics (all four dissipation terms, 8
    tracers, velocity noise) on a 48x48x16 mesh, 10 LSRK5 steps."""
    wl = WORKLOADS["lsrk5_512x512"].scaled(nx=48, ny=48, nlayers=16)
    (h, vn, tr), (rh, rvn, rtr) = _oracle_vs_gpu(wl, 10)
    assert rel_diff(h, rh) <= TOL
    assert rel_diff(vn, rvn) <= TOL
    assert rel_diff(tr, rtr) <= TOL


@pytest.mark.parametrize("K,T", [(1, 0), (3, 2), (33, 1), (70, 3)])
def test_uneven_levels_and_tracers(K, T):
    """Level counts that do not fill warps and tracer counts 0..3."""
    wl = WORKLOADS["lsrk5_512x512"].scaled(nx=12, ny=10, nlayers=K,
                                           ntracers=T)
    (h, vn, tr), (rh, rvn, rtr) = _oracle_vs_gpu(wl, 3, use_graph=False)
    assert rel_diff(h, rh) <= TOL
    assert rel_diff(vn, rvn) <= TOL
    assert rel_diff(tr, rtr) <= TOL


def test_increment_mode_adds():
    g = load_golden("rk4_all_terms")
    cfg = g["cfg"]
    mesh, params, model = gpu_setup(cfg)
    state = og.ShallowWaterState(mesh, params)
    state.upload(g["in_h"], g["in_vn"], g["in_tr"])
    tend = og.ShallowWaterState(mesh, params)
    model.compute_tendency(tend, state, 0.0, og.AddMode.replace)
    model.compute_tendency(tend, state, 0.0, og.AddMode.increment)
    th, tv, tt = tend.download()
    assert rel_diff(th, 2 * g["tend_h"]) <= TOL
    assert rel_diff(tv, 2 * g["tend_vn"]) <= TOL
    assert rel_diff(tt, 2 * g["tend_tr"]) <= TOL


def test_graph_and_direct_launches_agree_bitwise():
    wl = WORKLOADS["lsrk5_512x512"].scaled(nx=32, ny=32, nlayers=8,
                                           ntracers=2)
    outs = []
    for use_graph in (False, True, True):
        cfg = dict(nx=wl.nx, ny=wl.ny, dc=wl.dc, K=wl.nlayers, T=wl.ntracers,
                   f0=wl.f0, grav=wl.grav, visc_del2=wl.visc_del2,
                   visc_del4=wl.visc_del4, eddy_diff2=wl.eddy_diff2,
                   eddy_diff4=wl.eddy_diff4, disable_h=False,
                   disable_vn=False)
        mesh, params, model = gpu_setup(cfg)
        state = og.ShallowWaterState(mesh, params)
        state.upload(*initial_state(mesh, wl))
        st = og.LSRKStepper(model, 5)
        st.step(state, 0.0, wl.dt, 4, use_graph=use_graph)
        outs.append(state.download())
    for a, b in zip(outs[0], outs[1]):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(outs[1], outs[2]):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("nsteps", [1, 10])
def test_full_size_512x512_against_oracle(nsteps):
    """The full 512x512x64, 8-tracer LSRK5 workload (the benchmarked one):
    1 and 10 steps on the GPU against the oracle (all host cores, about 3 s
    a step), <= 1e-12."""
    wl = WORKLOADS["lsrk5_512x512"]
    (h, vn, tr), (rh, rvn, rtr) = _oracle_vs_gpu(wl, nsteps)
    assert rel_diff(h, rh) <= TOL
    assert rel_diff(vn, rvn) <= TOL
    assert rel_diff(tr, rtr) <= TOL


def test_full_size_conservation():
    """Size-independent properties at the full 512x512x64x8 size over 3
    LSRK5 steps: total thickness and every tracer's total are conserved to
    round-off (all transport and diffusion terms are in flux form)."""
    wl = WORKLOADS["lsrk5_512x512"]
    cfg = dict(nx=wl.nx, ny=wl.ny, dc=wl.dc, K=wl.nlayers, T=wl.ntracers,
               f0=wl.f0, grav=wl.grav, visc_del2=wl.visc_del2,
               visc_del4=wl.visc_del4, eddy_diff2=wl.eddy_diff2,
               eddy_diff4=wl.eddy_diff4, disable_h=False, disable_vn=False)
    mesh, params, model = gpu_setup(cfg)
    h0, vn0, tr0 = initial_state(mesh, wl)
    state = og.ShallowWaterState(mesh, params)
    state.upload(h0, vn0, tr0)
    m0 = og.mass_integral(state, model)
    og.LSRKStepper(model, 5).step(state, 0.0, wl.dt, 3)
    m1 = og.mass_integral(state, model)
    h, vn, tr = state.download()
    assert np.isfinite(h).all() and np.isfinite(vn).all() and np.isfinite(tr).all()
    assert abs(m1 - m0) <= 1e-14 * abs(m0)
    area = mesh.m_area_cell[:, None]
    for l in range(wl.ntracers):
        a0, a1 = np.sum(area * tr0[l]), np.sum(area * tr[l])
        assert abs(a1 - a0) <= 1e-13 * abs(a0)
