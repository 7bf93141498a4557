"""The linear shallow-water model and the opt-in bottom drag.

Both come from the reference's hierarchical source, which is never built
(shallow_water_hierarchical.cpp: LinearShallowWaterModel :676-775; the drag
term commented out at :479-486), so the oracle restates them and parity is
not pinned to a reference build.  What pins them besides the oracle:
- linear model: its TRiSK discretisation conserves energy exactly in the
  semi-discrete sense on the uniform hexagonal mesh (dE/dt = 0 to round-off),
  and it converges at second order to an exact plane gravity wave;
- drag: off unless asked for (the reference's live model ignores
  drag_coeff, so the default must equal a run without drag bit for bit), it
  touches only the lowest level, and it removes kinetic energy there.

Bounds: GPU vs oracle normwise relative <= 1e-12 (tendencies and 3 steps);
energy rate <= 1e-12 of the sum of its terms' magnitudes; observed order of
the plane-wave error within 0.15 of 2."""
import math

import numpy as np
import pytest

import omega_playground_gb300 as og
import pyoracle
from helpers import rel_diff
from omega_playground_gb300.workloads import uniform

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rand_state(mesh, T, seed, h0=1000.0):
    C_, E, K = mesh.m_ncells, mesh.m_nedges, mesh.m_nlayers
    h = h0 + uniform(seed, C_ * K).reshape(C_, K)
    vn = 0.2 * (uniform(seed + 1, E * K).reshape(E, K) - 0.5)
    tr = h[None] * uniform(seed + 2, T * C_ * K).reshape(T, C_, K)
    return h, vn, tr


def gpu_tendency(model, mesh, params, x, base=None, add_mode=0):
    S = og.ShallowWaterState(mesh, params)
    S.upload(*x)
    Tn = og.ShallowWaterState(mesh, params)
    if base is not None:
        Tn.upload(*base)
    else:
        Tn.fill(0.0)
    model.compute_tendency(Tn, S, 0.0, og.AddMode(add_mode))
    return Tn.download()


# ------------------------------------------------------------ linear ----

def linear_pair(nx, ny, K, h0=1000.0, f0=1e-4, **flags):
    mesh = og.PlanarHexagonalMesh(nx, ny, 1e4, K)
    params = og.LinearShallowWaterParams(m_f0=f0, m_h0=h0, **flags)
    model = og.LinearShallowWaterModel(mesh, params)
    om = pyoracle.OracleMesh(nx, ny, 1e4, K)
    omd = pyoracle.OracleModel(
        om, f0=f0, linear_h0=h0,
        disable_h_tendency=flags.get("m_disable_h_tendency", False),
        disable_vn_tendency=flags.get("m_disable_vn_tendency", False))
    return mesh, params, model, omd


@pytest.mark.parametrize("flags", [{}, {"m_disable_h_tendency": True},
                                   {"m_disable_vn_tendency": True}])
@pytest.mark.parametrize("add_mode", [0, 1])
def test_linear_tendency_matches_oracle(flags, add_mode):
    mesh, params, model, omd = linear_pair(12, 10, 5, **flags)
    x = rand_state(mesh, 0, 5)
    base = rand_state(mesh, 0, 9)
    want = omd.compute_tendency(x[0], x[1], None, add_mode=add_mode,
                                tend=tuple(a.copy() for a in base))
    got = gpu_tendency(model, mesh, params, x, base, add_mode)
    assert rel_diff(got[0], want[0]) <= TOL
    assert rel_diff(got[1], want[1]) <= TOL


@pytest.mark.parametrize("kind", ["rk4", "lsrk"])
def test_linear_steps_match_oracle(kind):
    mesh, params, model, omd = linear_pair(12, 10, 5)
    x = rand_state(mesh, 0, 21)
    ns = 4 if kind == "rk4" else 5
    want = omd.step(x[0].copy(), x[1].copy(), None, 0.0, 20.0, 3, kind=kind,
                    nstages=ns)
    S = og.ShallowWaterState(mesh, params)
    S.upload(*x)
    st = og.RK4Stepper(model) if kind == "rk4" else og.LSRKStepper(model, 5)
    st.step(S, 0.0, 20.0, 3)
    got = S.download()
    assert rel_diff(got[0], want[0]) <= TOL
    assert rel_diff(got[1], want[1]) <= TOL
    # energy integral with h0-weighted kinetic energy, as the oracle's
    e = og.energy_integral(S, model)
    assert abs(e - omd.energy(want[0], want[1])) <= TOL * abs(e)


def test_linear_semi_discrete_energy_is_conserved():
    """dE/dt = g sum_c A h h_t + h0 sum_e dv dc vn vn_t = 0 (TRiSK)."""
    mesh, params, model, _ = linear_pair(16, 14, 3, f0=1e-4)
    x = rand_state(mesh, 0, 31)
    ht, vt, _ = gpu_tendency(model, mesh, params, x)
    h, vn = x[0], x[1]
    A = mesh.m_area_cell[:, None]
    de = (mesh.m_dv_edge * mesh.m_dc_edge)[:, None]
    terms = np.concatenate([(params.m_grav * A * h * ht).ravel(),
                            (params.m_h0 * de * vn * vt).ravel()])
    assert abs(terms.sum()) <= TOL * np.abs(terms).sum()


def plane_wave_error(n, h0=1000.0, eta=1.0, g=9.81):
    """Max error of h after the same physical time against the exact plane
    gravity wave h = h0 + eta cos(k.x - w t), u = g eta k / w cos(...),
    w^2 = g h0 |k|^2 (f0 = 0)."""
    L = 6.4e5
    dc = L / n
    mesh = og.PlanarHexagonalMesh(n, n, dc, 1)
    params = og.LinearShallowWaterParams(m_f0=0.0, m_h0=h0, m_grav=g)
    model = og.LinearShallowWaterModel(mesh, params)
    Lx, Ly = mesh.m_period_x, mesh.m_period_y
    kx, ky = 2 * math.pi / Lx, 2 * math.pi / Ly
    w = math.sqrt(g * h0 * (kx * kx + ky * ky))

    def fields(t):
        ph_c = kx * mesh.m_x_cell + ky * mesh.m_y_cell - w * t
        ph_e = kx * mesh.m_x_edge + ky * mesh.m_y_edge - w * t
        a = g * eta / w * np.cos(ph_e)
        un = a * (kx * np.cos(mesh.m_angle_edge) + ky * np.sin(mesh.m_angle_edge))
        return (h0 + eta * np.cos(ph_c))[:, None], un[:, None]

    T = 0.25 * 2 * math.pi / w
    nsteps = int(math.ceil(T / (0.1 * dc / math.sqrt(g * h0))))
    dt = T / nsteps
    S = og.ShallowWaterState(mesh, params)
    S.upload(*fields(0.0))
    og.RK4Stepper(model).step(S, 0.0, dt, nsteps)
    h = S.download()[0]
    return float(np.max(np.abs(h - fields(T)[0])))


def test_linear_plane_wave_second_order():
    errs = [plane_wave_error(n) for n in (16, 32, 64)]
    rates = [math.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert all(abs(r - 2.0) <= 0.15 for r in rates), (errs, rates)


def test_linear_model_rejects_tracers_and_is_not_differentiated():
    mesh = og.PlanarHexagonalMesh(8, 8, 1e4, 2)
    with pytest.raises(og.SwgError):
        og.LinearShallowWaterModel(
            mesh, og.LinearShallowWaterParams(m_h0=1e3, m_ntracers=1))
    model = og.LinearShallowWaterModel(mesh, og.LinearShallowWaterParams(m_h0=1e3))
    with pytest.raises(og.SwgError):
        og.Adjoint(model, 4)


# -------------------------------------------------------------- drag ----

DRAG = dict(m_f0=1e-4, m_visc_del2=1e3, m_drag_coeff=2e-3, m_ntracers=1)


def drag_models(nx, ny, K):
    mesh = og.PlanarHexagonalMesh(nx, ny, 1e4, K)
    params = og.ShallowWaterParams(**DRAG)
    return (mesh, params, og.ShallowWaterModel(mesh, params),
            og.ShallowWaterModel(mesh, params, apply_drag=True))


def oracle_drag(nx, ny, K, apply_drag):
    om = pyoracle.OracleMesh(nx, ny, 1e4, K)
    return pyoracle.OracleModel(om, f0=DRAG["m_f0"], visc_del2=DRAG["m_visc_del2"],
                                ntracers=1, drag_coeff=DRAG["m_drag_coeff"],
                                apply_drag=apply_drag)


def test_drag_is_off_by_default_like_the_reference():
    mesh, params, plain, _ = drag_models(10, 8, 4)
    nodrag = og.ShallowWaterModel(mesh, og.ShallowWaterParams(
        **dict(DRAG, m_drag_coeff=0.0)))
    x = rand_state(mesh, 1, 41)
    a = gpu_tendency(plain, mesh, params, x)
    b = gpu_tendency(nodrag, mesh, params, x)
    for u, v in zip(a, b):
        np.testing.assert_array_equal(u, v)


def test_drag_tendency_and_steps_match_oracle():
    nx, ny, K = 10, 8, 4
    mesh, params, plain, drag = drag_models(nx, ny, K)
    omd = oracle_drag(nx, ny, K, True)
    x = rand_state(mesh, 1, 43)
    want = omd.compute_tendency(*x)
    got = gpu_tendency(drag, mesh, params, x)
    for g_, w_ in zip(got, want):
        assert rel_diff(g_, w_) <= TOL
    # only the lowest level differs from the model without drag
    ref = gpu_tendency(plain, mesh, params, x)
    np.testing.assert_array_equal(got[1][:, :K - 1], ref[1][:, :K - 1])
    assert np.any(got[1][:, K - 1] != ref[1][:, K - 1])
    # and it opposes the bottom flow: sum_e dv dc vn * (drag term) < 0
    dterm = got[1][:, K - 1] - ref[1][:, K - 1]
    assert float(np.sum(mesh.m_dv_edge * mesh.m_dc_edge * x[1][:, K - 1] *
                        dterm)) < 0
    S = og.ShallowWaterState(mesh, params)
    S.upload(*x)
    og.RK4Stepper(drag).step(S, 0.0, 20.0, 3)
    want = omd.step(*(a.copy() for a in x), 0.0, 20.0, 3, kind="rk4",
                    nstages=4)
    for g_, w_ in zip(S.download(), want):
        assert rel_diff(g_, w_) <= TOL
