"""The product's host mesh builder (swg_planar_hex_mesh_build, pure host
code) reproduces PlanarHexagonalMesh bit for bit: checked against the oracle
(itself pinned to the reference) and the golden fixtures, on even, odd and
rectangular meshes."""
import ctypes as C

import numpy as np
import pytest

import pyoracle
from helpers import golden_names, load_golden
from omega_playground_gb300 import _capi


def product_tables(nx, ny, dc):
    sizes = {"C": nx * ny, "E": 3 * nx * ny, "V": 2 * nx * ny}
    ht, tabs = _capi.HexTables(), {}
    for name, (ent, w) in _capi.HEX_SHAPE.items():
        dt = np.int32 if name in _capi.HEX_INT else np.float64
        tabs[name] = np.zeros((sizes[ent], w) if w > 1 else (sizes[ent],), dt)
        ct = C.c_int if dt == np.int32 else C.c_double
        setattr(ht, name, tabs[name].ctypes.data_as(C.POINTER(ct)))
    px, py = C.c_double(), C.c_double()
    _capi.check(_capi.lib().swg_planar_hex_mesh_build(
        nx, ny, dc, C.byref(ht), C.byref(px), C.byref(py)))
    return tabs, px.value, py.value


@pytest.mark.parametrize("nx,ny,dc", [(1, 1, 1e4), (1, 2, 1e4), (2, 1, 1e4),
                                      (2, 3, 1e4), (2, 2, 1.0), (4, 4, 1e4),
                                      (5, 7, 1e4),
                                      (6, 10, 2e4), (16, 16, 1e4),
                                      (25, 29, 2e5), (64, 64, 1e4),
                                      (7, 6, 0.125)])
def test_matches_oracle(nx, ny, dc):
    tabs, px, py = product_tables(nx, ny, dc)
    m = pyoracle.OracleMesh(nx, ny, dc, 1)
    for k, v in tabs.items():
        np.testing.assert_array_equal(v, m.tables[k], err_msg=k)
    assert px == m.period_x and py == m.period_y


@pytest.mark.parametrize("name", golden_names())
def test_matches_golden(name):
    g = load_golden(name)
    cfg = g["cfg"]
    tabs, _, _ = product_tables(cfg["nx"], cfg["ny"], cfg["dc"])
    for k, v in tabs.items():
        if k in g:
            np.testing.assert_array_equal(v, g[k], err_msg=k)


def test_rejects_degenerate_sizes():
    tabs = _capi.HexTables()
    for nx, ny in ((0, 4), (3, 0), (-1, 2)):
        rc = _capi.lib().swg_planar_hex_mesh_build(nx, ny, 1.0, C.byref(tabs),
                                                   None, None)
        assert rc == 1
        assert b"nx >= 1" in _capi.lib().swg_last_error()


def test_operator_convergence_on_tables():
    """operator_convergence.cpp:226-301 on the product's tables (host numpy):
    gradient, divergence and TRiSK reconstruction converge at rate 2 and the
    curl at rate 1 (L-infinity, +-0.05)."""
    errs = {"grad": [], "div": [], "curl": [], "recon": []}
    nx = 6
    for _ in range(5):
        t, Lx, Ly = product_tables(nx, nx, 1.0 / nx)
        xe, ye, ang = t["x_edge"], t["y_edge"], t["angle_edge"]
        nxv, nyv = np.cos(ang), np.sin(ang)
        xc, yc = t["x_cell"], t["y_cell"]
        tw = 2 * np.pi
        f = np.sin(tw * xc / Lx) * np.sin(tw * yc / Ly)
        coe = t["cells_on_edge"]
        grad = (f[coe[:, 1]] - f[coe[:, 0]]) / t["dc_edge"]
        gx = tw / Lx * np.cos(tw * xe / Lx) * np.sin(tw * ye / Ly)
        gy = tw / Ly * np.sin(tw * xe / Lx) * np.cos(tw * ye / Ly)
        errs["grad"].append(np.max(np.abs(nxv * gx + nyv * gy - grad)))
        vx = np.sin(tw * xe / Lx) * np.cos(tw * ye / Ly)
        vy = np.cos(tw * xe / Lx) * np.sin(tw * ye / Ly)
        u = nxv * vx + nyv * vy
        eoc = t["edges_on_cell"]
        div = np.sum(t["dv_edge"][eoc] * t["edge_sign_on_cell"] * u[eoc],
                     axis=1) / t["area_cell"]
        ediv = tw * (1 / Lx + 1 / Ly) * np.cos(tw * xc / Lx) * np.cos(tw * yc / Ly)
        errs["div"].append(np.max(np.abs(ediv - div)))
        eov = t["edges_on_vertex"]
        curl = np.sum(t["dc_edge"][eov] * t["edge_sign_on_vertex"] * u[eov],
                      axis=1) / t["area_triangle"]
        xv, yv = t["x_vertex"], t["y_vertex"]
        ecurl = tw * (-1 / Lx + 1 / Ly) * np.sin(tw * xv / Lx) * np.sin(tw * yv / Ly)
        errs["curl"].append(np.max(np.abs(ecurl - curl)))
        eoe = t["edges_on_edge"][:, :10]
        rec = np.sum(t["weights_on_edge"][:, :10] * u[eoe], axis=1)
        erec = -nyv * vx + nxv * vy
        errs["recon"].append(np.max(np.abs(erec - rec)))
        nx *= 2
    for name, expect in (("grad", 2), ("div", 2), ("curl", 1), ("recon", 2)):
        e = errs[name]
        rate = np.log2(e[-2] / e[-1])
        assert abs(rate - expect) < 0.05, (name, e, rate)


def test_odd_row_seam_flag():
    """Odd ny is flagged on the mesh classes (the reference races there)."""
    from omega_playground_gb300.shallow_water import PlanarHexagonalMesh
    assert PlanarHexagonalMesh.odd_row_seam.fget(
        type("M", (), {"m_ny": 29})())
    assert not PlanarHexagonalMesh.odd_row_seam.fget(
        type("M", (), {"m_ny": 28})())


def test_every_small_size_matches_oracle():
    """Every nx, ny in 1..12 (odd and even rows, one-cell-wide meshes):
    the product's builder against the oracle, bit for bit."""
    for nx in range(1, 13):
        for ny in range(1, 13):
            tabs, px, py = product_tables(nx, ny, 1e4)
            m = pyoracle.OracleMesh(nx, ny, 1e4, 1)
            for k, v in tabs.items():
                np.testing.assert_array_equal(v, m.tables[k],
                                              err_msg=f"{nx}x{ny} {k}")
            assert px == m.period_x and py == m.period_y
