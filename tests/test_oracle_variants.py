"""The oracle's restatements of the linear model and the opt-in bottom drag
(shallow_water_hierarchical.cpp:676-775 and :479-486, which the reference
never builds), pinned by properties instead of a reference build:
- linear model: semi-discrete energy conservation of its TRiSK operators on
  the uniform hexagonal mesh, and second-order convergence to an exact plane
  gravity wave;
- drag: the default model ignores drag_coeff (as the reference's live model
  does), the drag only changes the lowest level and removes kinetic energy
  there."""
import math

import numpy as np
import pytest

import pyoracle
from omega_playground_gb300.workloads import uniform


def rand_state(om, T, seed, h0=1000.0):
    C_, E, K = om.ncells, om.nedges, om.nlayers
    h = h0 + uniform(seed, C_ * K).reshape(C_, K)
    vn = 0.2 * (uniform(seed + 1, E * K).reshape(E, K) - 0.5)
    tr = h[None] * uniform(seed + 2, T * C_ * K).reshape(T, C_, K)
    return h, vn, tr


def test_oracle_linear_energy_rate_is_zero():
    om = pyoracle.OracleMesh(16, 14, 1e4, 3)
    md = pyoracle.OracleModel(om, f0=1e-4, linear_h0=1000.0)
    h, vn, tr = rand_state(om, 0, 31)
    ht, vt, _ = md.compute_tendency(h, vn, tr)
    A = om.area_cell[:, None]
    de = (om.dv_edge * om.dc_edge)[:, None]
    terms = np.concatenate([(9.81 * A * h * ht).ravel(),
                            (1000.0 * de * vn * vt).ravel()])
    assert abs(terms.sum()) <= 1e-12 * np.abs(terms).sum()


def oracle_plane_wave_error(n, h0=1000.0, eta=1.0, g=9.81):
    L = 6.4e5
    dc = L / n
    om = pyoracle.OracleMesh(n, n, dc, 1)
    md = pyoracle.OracleModel(om, f0=0.0, grav=g, linear_h0=h0)
    kx, ky = 2 * math.pi / om.period_x, 2 * math.pi / om.period_y
    w = math.sqrt(g * h0 * (kx * kx + ky * ky))

    def fields(t):
        ph_c = kx * om.x_cell + ky * om.y_cell - w * t
        ph_e = kx * om.x_edge + ky * om.y_edge - w * t
        a = g * eta / w * np.cos(ph_e)
        un = a * (kx * np.cos(om.angle_edge) + ky * np.sin(om.angle_edge))
        return (h0 + eta * np.cos(ph_c))[:, None].copy(), un[:, None].copy()

    T = 0.25 * 2 * math.pi / w
    nsteps = int(math.ceil(T / (0.1 * dc / math.sqrt(g * h0))))
    h, vn = fields(0.0)
    md.step(h, vn, None, 0.0, T / nsteps, nsteps, kind="rk4", nstages=4)
    return float(np.max(np.abs(h - fields(T)[0])))


def test_oracle_linear_plane_wave_second_order():
    errs = [oracle_plane_wave_error(n) for n in (16, 32, 64)]
    rates = [math.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert all(abs(r - 2.0) <= 0.15 for r in rates), (errs, rates)


@pytest.mark.parametrize("apply_drag", [False, True])
def test_oracle_drag(apply_drag):
    om = pyoracle.OracleMesh(10, 8, 1e4, 4)
    kw = dict(f0=1e-4, visc_del2=1e3, ntracers=1)
    ref = pyoracle.OracleModel(om, **kw)
    md = pyoracle.OracleModel(om, drag_coeff=2e-3, apply_drag=apply_drag, **kw)
    x = rand_state(om, 1, 43)
    a = ref.compute_tendency(*x)
    b = md.compute_tendency(*x)
    if not apply_drag:  # the coefficient alone changes nothing
        for u, v in zip(a, b):
            np.testing.assert_array_equal(u, v)
        return
    K = om.nlayers
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1][:, :K - 1], b[1][:, :K - 1])
    d = b[1][:, K - 1] - a[1][:, K - 1]
    assert float(np.sum(om.dv_edge * om.dc_edge * x[1][:, K - 1] * d)) < 0
