"""The model's tendency-term members and their m_enabled switches
(shallow_water_model.hpp:19-29, read at compute time by
shallow_water_model.cpp:43-311), against the oracle with the same term
switched off.

Bounds: tendencies and 3 LSRK5 steps <= 1e-12 normwise relative; switching
a term back on, or switching nothing, is bitwise neutral."""
import numpy as np
import pytest

import omega_playground_gb300 as og
import pyoracle
from helpers import rel_diff
from omega_playground_gb300.shallow_water import TERMS
from omega_playground_gb300.workloads import uniform

pytestmark = pytest.mark.gpu

TOL = 1e-12
COEF = dict(f0=1e-4, grav=9.81, visc_del2=1e3, visc_del4=1e9, eddy_diff2=1e3,
            eddy_diff4=1e9)
NX, NY, K, T = 12, 10, 5, 2


def setup():
    mesh = og.PlanarHexagonalMesh(NX, NY, 1e4, K)
    params = og.ShallowWaterParams(
        m_f0=COEF["f0"], m_grav=COEF["grav"], m_visc_del2=COEF["visc_del2"],
        m_visc_del4=COEF["visc_del4"], m_eddy_diff2=COEF["eddy_diff2"],
        m_eddy_diff4=COEF["eddy_diff4"], m_ntracers=T)
    om = pyoracle.OracleMesh(NX, NY, 1e4, K)
    return (mesh, params, og.ShallowWaterModel(mesh, params),
            pyoracle.OracleModel(om, ntracers=T, **COEF))


def state(mesh, seed):
    C_, E = mesh.m_ncells, mesh.m_nedges
    h = 1000.0 + 5.0 * uniform(seed, C_ * K).reshape(C_, K)
    vn = 0.2 * (uniform(seed + 1, E * K).reshape(E, K) - 0.5)
    tr = h[None] * (1.0 + uniform(seed + 2, T * C_ * K).reshape(T, C_, K))
    return h, vn, tr


def gpu_tendency(model, mesh, params, x, base, add_mode):
    S = og.ShallowWaterState(mesh, params)
    S.upload(*x)
    Tn = og.ShallowWaterState(mesh, params)
    Tn.upload(*base)
    model.compute_tendency(Tn, S, 0.0, og.AddMode(add_mode))
    return Tn.download()


@pytest.mark.parametrize("term", range(len(TERMS)))
@pytest.mark.parametrize("add_mode", [0, 1])
def test_each_term_off_matches_oracle(term, add_mode):
    mesh, params, model, omd = setup()
    getattr(model, TERMS[term]).m_enabled = False
    assert not getattr(model, TERMS[term]).m_enabled
    omd.set_term(term, False)
    x, base = state(mesh, 3), state(mesh, 9)
    want = omd.compute_tendency(*x, add_mode=add_mode,
                                tend=tuple(a.copy() for a in base))
    got = gpu_tendency(model, mesh, params, x, base, add_mode)
    for g, w in zip(got, want):
        assert rel_diff(g, w) <= TOL, TERMS[term]
    # and the switch did something
    on = og.ShallowWaterModel(mesh, params)
    ref = gpu_tendency(on, mesh, params, x, base, add_mode)
    assert any(np.any(a != b) for a, b in zip(got, ref))


def test_all_terms_off_replace_zeroes_and_increment_keeps():
    mesh, params, model, _ = setup()
    for name in TERMS:
        getattr(model, name).m_enabled = False
    x, base = state(mesh, 5), state(mesh, 6)
    for a in gpu_tendency(model, mesh, params, x, base, 0):
        np.testing.assert_array_equal(a, 0.0)
    for a, b in zip(gpu_tendency(model, mesh, params, x, base, 1), base):
        np.testing.assert_array_equal(a, b)


def test_switching_back_is_bitwise_neutral():
    mesh, params, model, _ = setup()
    x, base = state(mesh, 7), state(mesh, 8)
    ref = gpu_tendency(model, mesh, params, x, base, 0)
    for name in TERMS:
        getattr(model, name).m_enabled = False
        getattr(model, name).m_enabled = True
    for a, b in zip(gpu_tendency(model, mesh, params, x, base, 0), ref):
        np.testing.assert_array_equal(a, b)


def test_stepper_follows_a_switch_and_matches_oracle():
    """A stepper captured its step graph with every term on; after the PV
    flux and the tracer del2 are switched off, its graph path equals direct
    launches and the oracle's LSRK5 steps with the same terms off."""
    mesh, params, model, omd = setup()
    x = state(mesh, 11)
    st = og.LSRKStepper(model, 5)
    S = og.ShallowWaterState(mesh, params)
    S.upload(*x)
    st.step(S, 0.0, 20.0, 2)                      # graph captured, all on
    model.m_pv_flux_edge.m_enabled = False
    model.m_tracer_diff_cell.m_enabled = False
    omd.set_term(1, False)
    omd.set_term(7, False)
    S.upload(*x)
    st.step(S, 0.0, 20.0, 3)                      # graph path again
    got = S.download()
    D = og.ShallowWaterState(mesh, params)
    D.upload(*x)
    og.LSRKStepper(model, 5).step(D, 0.0, 20.0, 3, use_graph=False)
    for a, b in zip(got, D.download()):
        np.testing.assert_array_equal(a, b)
    want = omd.step(*(a.copy() for a in x), 0.0, 20.0, 3, kind="lsrk",
                    nstages=5)
    for a, b in zip(got, want):
        assert rel_diff(a, b) <= TOL


def test_enabling_a_zero_coefficient_term_is_an_error():
    mesh = og.PlanarHexagonalMesh(8, 8, 1e4, 2)
    params = og.ShallowWaterParams(m_f0=1e-4, m_visc_del2=1e3)
    model = og.ShallowWaterModel(mesh, params)
    assert model.m_vel_diff_edge.m_enabled
    assert not model.m_vel_hyperdiff_edge.m_enabled
    with pytest.raises(og.SwgError):
        model.m_vel_hyperdiff_edge.m_enabled = True
    model.m_ke_grad_edge.m_enabled = False
    og.Adjoint(model, 4)                           # switched terms differentiate


def test_beta_plane_f_vertex_matches_oracle():
    """The model's m_f_vertex (f0 after construction) written with a beta
    plane f = f0 + beta (y - Ly/2) on both sides: tendencies and three RK4
    steps (graph path) <= 1e-12, and the field reads back."""
    mesh, params, model, omd = setup()
    np.testing.assert_array_equal(model.m_f_vertex, COEF["f0"])
    om = omd.mesh
    f = COEF["f0"] + 1.6e-11 * (om.y_vertex - 0.5 * om.period_y)
    model.m_f_vertex = f
    omd.set_f_vertex(f)
    np.testing.assert_array_equal(model.m_f_vertex, f)
    x, base = state(mesh, 21), state(mesh, 22)
    want = omd.compute_tendency(*x, tend=tuple(a.copy() for a in base))
    got = gpu_tendency(model, mesh, params, x, base, 0)
    for g, w in zip(got, want):
        assert rel_diff(g, w) <= TOL
    flat = gpu_tendency(og.ShallowWaterModel(mesh, params), mesh, params, x,
                        base, 0)
    assert np.any(got[1] != flat[1])              # vn feels the beta plane
    S = og.ShallowWaterState(mesh, params)
    S.upload(*x)
    og.RK4Stepper(model).step(S, 0.0, 20.0, 3)
    want = omd.step(*(a.copy() for a in x), 0.0, 20.0, 3, kind="rk4",
                    nstages=4)
    for g, w in zip(S.download(), want):
        assert rel_diff(g, w) <= TOL


def test_switch_between_adjoint_forward_and_backward_is_an_error():
    """The reverse sweep re-runs plain steps with the model's current terms
    and replays the tape captured with the forward's: a switch in between
    is refused; switching back restores the forward's set.  The tendency-
    level calls differentiate the current set."""
    mesh, params, model, _ = setup()
    adj = og.Adjoint(model, 2)
    x = state(mesh, 31)
    X = og.ShallowWaterState(mesh, params)
    X.upload(*x)
    XN = og.ShallowWaterState(mesh, params)
    adj.forward(X, 0.0, 20.0, 4, XN)
    model.m_ke_grad_edge.m_enabled = False
    LAM = og.ShallowWaterState(mesh, params)
    LAM.upload(*state(mesh, 32))
    with pytest.raises(og.SwgError, match="switched"):
        adj.backward(LAM)
    W = og.ShallowWaterState(mesh, params)
    adj.adj_tendency(X, LAM, W)
    adj.tlm_tendency(X, LAM, W)
    model.m_ke_grad_edge.m_enabled = True
    adj.backward(LAM)


def test_adjoint_with_beta_plane_f_vertex_dot_product():
    """A written m_f_vertex enters the taped PV and its adjoint: tendency
    and trajectory dot products against the tangent-linear model <= 1e-12."""
    mesh, params, model, omd = setup()
    om = omd.mesh
    model.m_f_vertex = COEF["f0"] + 1.6e-11 * (om.y_vertex - 0.5 * om.period_y)
    adj = og.Adjoint(model, 2)
    x = state(mesh, 41)
    dx = tuple(1e-3 * (uniform(50 + j, a.size).reshape(a.shape) - 0.5)
               for j, a in enumerate(x))
    mu = tuple(uniform(60 + j, a.size).reshape(a.shape) - 0.5
               for j, a in enumerate(x))

    def mk(a):
        st = og.ShallowWaterState(mesh, params)
        st.upload(*a)
        return st

    def dot(a, b):
        return sum(float(np.sum(p * q)) for p, q in zip(a, b))

    X = mk(x)
    JD, JT = og.ShallowWaterState(mesh, params), og.ShallowWaterState(mesh, params)
    adj.tlm_tendency(X, mk(dx), JD)
    adj.adj_tendency(X, mk(mu), JT)
    lhs, rhs = dot(JD.download(), mu), dot(dx, JT.download())
    assert abs(lhs - rhs) <= TOL * max(abs(lhs), abs(rhs)), (lhs, rhs)
    XN = og.ShallowWaterState(mesh, params)
    adj.forward(X, 0.0, 20.0, 5, XN)
    LAM = mk(mu)
    adj.backward(LAM)
    DX = mk(dx)
    adj.tlm_apply(X, DX, 0.0, 20.0, 5)
    lhs, rhs = dot(DX.download(), mu), dot(dx, LAM.download())
    assert abs(lhs - rhs) <= TOL * max(abs(lhs), abs(rhs)), (lhs, rhs)


@pytest.mark.parametrize("stepper,nstages", [("rk4", 4), ("lsrk", 5)])
@pytest.mark.parametrize("term", range(len(TERMS)))
def test_adjoint_with_a_term_switched_off(term, stepper, nstages):
    """Each of the nine terms switched off alone: the adjoint tendency and a
    5-step trajectory (3 snapshots) against the tangent-linear model of the
    same switched model, dot products <= 1e-12, and the forward sweep's x_N
    equal to the switched stepper's bit for bit."""
    mesh, params, model, _ = setup()
    getattr(model, TERMS[term]).m_enabled = False
    adj = og.Adjoint(model, 3, stepper, nstages)
    x = state(mesh, 71)
    dx = tuple(1e-3 * (uniform(80 + j, a.size).reshape(a.shape) - 0.5)
               for j, a in enumerate(x))
    mu = tuple(uniform(90 + j, a.size).reshape(a.shape) - 0.5
               for j, a in enumerate(x))

    def mk(a):
        st = og.ShallowWaterState(mesh, params)
        st.upload(*a)
        return st

    def dot(a, b):
        return sum(float(np.sum(p * q)) for p, q in zip(a, b))

    X = mk(x)
    JD, JT = og.ShallowWaterState(mesh, params), og.ShallowWaterState(mesh, params)
    adj.tlm_tendency(X, mk(dx), JD)
    adj.adj_tendency(X, mk(mu), JT)
    lhs, rhs = dot(JD.download(), mu), dot(dx, JT.download())
    assert abs(lhs - rhs) <= TOL * max(abs(lhs), abs(rhs)), (lhs, rhs)
    XN = og.ShallowWaterState(mesh, params)
    adj.forward(X, 0.0, 20.0, 5, XN)
    LAM = mk(mu)
    adj.backward(LAM)
    DX = mk(dx)
    adj.tlm_apply(X, DX, 0.0, 20.0, 5)
    lhs, rhs = dot(DX.download(), mu), dot(dx, LAM.download())
    assert abs(lhs - rhs) <= TOL * max(abs(lhs), abs(rhs)), (lhs, rhs)
    ref = mk(x)
    (og.RK4Stepper(model) if stepper == "rk4"
     else og.LSRKStepper(model, nstages)).step(ref, 0.0, 20.0, 5,
                                               use_graph=False)
    for a, b in zip(XN.download(), ref.download()):
        np.testing.assert_array_equal(a, b)
