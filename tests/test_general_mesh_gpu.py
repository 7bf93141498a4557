"""General MPAS mesh input against the oracle: tables that are not a regular
hexagonal mesh.

The planar hexagonal tables are perturbed in place (the oracle reads the same
arrays): random cell, edge, triangle and kite geometry; cells with 5 edges;
edges with fewer edges-on-edge entries; TRiSK weights where the hexagon has
zeros (10 nonzero weights per edge); edges with dv < dc/4 (the del4
Laplacian's 1/max(dv, dc/4) differs from 1/dv); random mesh_scaling_del2/4, a
random 0/1 edge_mask and random per-column max levels for the diagnostics.
The connectivity stays a valid mesh, so every index is in range.

Bounds (normwise relative): tendencies and states after 3 steps <= 1e-12;
diagnostics <= 1e-12 relative; adjoint dot products <= 1e-12."""
import numpy as np
import pytest

import omega_playground_gb300 as og
import pyoracle
from helpers import rel_diff
from omega_playground_gb300.workloads import uniform

pytestmark = pytest.mark.gpu

TOL = 1e-12
TABLES = ("nedges_on_cell", "edges_on_cell", "nedges_on_edge",
          "edges_on_edge", "cells_on_edge", "vertices_on_edge",
          "edges_on_vertex", "cells_on_vertex", "area_cell",
          "edge_sign_on_cell", "dc_edge", "dv_edge", "weights_on_edge",
          "area_triangle", "kiteareas_on_vertex", "edge_sign_on_vertex")


def general_mesh(nx, ny, K, seed, adjoint_ready=False, cut_cells=None):
    """Perturbed tables; with adjoint_ready the edge mask stays all ones,
    every dv stays >= dc/4 and every cell keeps its 6 edges (the adjoint's
    supported set: cutting a cell's list to 5 leaves an edge its neighbour
    still lists, which no consistent mesh has and the adjoint rejects)."""
    om = pyoracle.OracleMesh(nx, ny, 1e4, K)
    t = om.tables
    C_, E, V = om.ncells, om.nedges, om.nvertices

    def jitter(a, s, amp=0.2):
        a *= 1.0 + amp * (uniform(s, a.size).reshape(a.shape) - 0.5)

    jitter(t["area_cell"], seed + 1)
    jitter(t["dc_edge"], seed + 2)
    jitter(t["dv_edge"], seed + 3)
    jitter(t["area_triangle"], seed + 4)
    jitter(t["kiteareas_on_vertex"], seed + 5)
    jitter(t["weights_on_edge"], seed + 6)
    u = uniform(seed + 7, E)
    if not adjoint_ready:
        t["dv_edge"][u < 0.05] = 0.2 * t["dc_edge"][u < 0.05]
    u = uniform(seed + 8, C_)
    if (not adjoint_ready) if cut_cells is None else cut_cells:
        t["nedges_on_cell"][u < 0.1] = 5
    u = uniform(seed + 9, E)
    w = t["weights_on_edge"]
    for e in np.nonzero(u < 0.1)[0]:      # fill the hexagon's zero weights
        n = t["nedges_on_edge"][e]
        zero = np.nonzero(w[e, :n] == 0.0)[0]
        w[e, zero] = 0.05 * (1.0 + u[e])
    t["nedges_on_edge"][(u > 0.9) & (u < 0.95)] = 7
    t["mesh_scaling_del2"][:] = 0.5 + uniform(seed + 10, E)
    t["mesh_scaling_del4"][:] = 0.5 + uniform(seed + 11, E)
    if not adjoint_ready:
        t["edge_mask"][:] = (uniform(seed + 12, E * K) < 0.8).reshape(E, K)
    mlc = (1 + uniform(seed + 13, C_) * K).astype(np.int32)
    mlv = (uniform(seed + 14, V) * (K + 1)).astype(np.int32)
    om.set_max_levels(np.minimum(mlc, K), np.minimum(mlv, K))
    gm = og.MPASMesh.from_tables(
        {n: t[n] for n in TABLES}, K,
        mesh_scaling_del2=t["mesh_scaling_del2"],
        mesh_scaling_del4=t["mesh_scaling_del4"], edge_mask=t["edge_mask"],
        max_level_cell=om.max_level_cell,
        max_level_vertex_bot=om.max_level_vertex_bot)
    return om, gm


PARAMS = dict(f0=1e-4, grav=9.81, visc_del2=1e3, visc_del4=1e9,
              eddy_diff2=1e3, eddy_diff4=1e9)


def models(om, gm, T, **over):
    p = dict(PARAMS, **over)
    omd = pyoracle.OracleModel(om, ntracers=T, **p)
    gp = og.ShallowWaterParams(
        m_f0=p["f0"], m_grav=p["grav"], m_visc_del2=p["visc_del2"],
        m_visc_del4=p["visc_del4"], m_eddy_diff2=p["eddy_diff2"],
        m_eddy_diff4=p["eddy_diff4"], m_ntracers=T)
    return omd, gp, og.ShallowWaterModel(gm, gp)


def state(om, T, seed):
    C_, E, K = om.ncells, om.nedges, om.nlayers
    h = 1000.0 + uniform(seed, C_ * K).reshape(C_, K)
    vn = 0.1 * (uniform(seed + 1, E * K).reshape(E, K) - 0.5)
    tr = h[None] * uniform(seed + 2, T * C_ * K).reshape(T, C_, K)
    return h, vn, tr


@pytest.mark.parametrize("nx,ny,K,T", [(10, 8, 7, 2), (6, 6, 33, 1)])
@pytest.mark.parametrize("add_mode", [0, 1])
def test_general_mesh_tendency(nx, ny, K, T, add_mode):
    om, gm = general_mesh(nx, ny, K, 4242 + nx)
    omd, gp, model = models(om, gm, T)
    x = state(om, T, 77)
    base = state(om, T, 99)  # prior tendency for the increment mode
    want = omd.compute_tendency(*x, t=0.0, add_mode=add_mode,
                                tend=tuple(a.copy() for a in base))
    S = og.ShallowWaterState(gm, gp)
    S.upload(*x)
    Tn = og.ShallowWaterState(gm, gp)
    Tn.upload(*base)
    model.compute_tendency(Tn, S, 0.0, og.AddMode(add_mode))
    for got, ref in zip(Tn.download(), want):
        assert rel_diff(got, ref) <= TOL


@pytest.mark.parametrize("kind", ["rk4", "lsrk"])
def test_general_mesh_steps(kind):
    om, gm = general_mesh(10, 8, 7, 5151)
    T = 2
    omd, gp, model = models(om, gm, T)
    x = state(om, T, 31)
    dt = 5.0
    want = omd.step(*(a.copy() for a in x), 0.0, dt, 3, kind=kind,
                    nstages=4 if kind == "rk4" else 5)
    S = og.ShallowWaterState(gm, gp)
    S.upload(*x)
    st = og.RK4Stepper(model) if kind == "rk4" else og.LSRKStepper(model, 5)
    st.step(S, 0.0, dt, 3)
    for got, ref in zip(S.download(), want):
        assert rel_diff(got, ref) <= TOL


def test_general_mesh_diagnostics_with_max_levels():
    om, gm = general_mesh(10, 8, 9, 6161)
    omd, gp, model = models(om, gm, 0)
    h, vn, _ = state(om, 0, 13)
    S = og.ShallowWaterState(gm, gp)
    S.upload(h, vn, None)
    for got, ref in ((og.mass_integral(S, model), omd.mass(h)),
                     (og.energy_integral(S, model), omd.energy(h, vn)),
                     (og.circulation_integral(S, model), omd.circulation(vn))):
        assert abs(got - ref) <= TOL * abs(ref), (got, ref)
    # the max levels matter: the full-column sums differ
    assert abs(og.mass_integral(S, model) - float(
        np.sum(om.area_cell[:, None] * h))) > 1e-6 * abs(omd.mass(h))


@pytest.mark.parametrize("full", [False, True])
@pytest.mark.parametrize("stepper,nstages", [("rk4", 4), ("lsrk", 5)])
def test_general_mesh_adjoint_dot_products(stepper, nstages, full):
    """The adjoint on perturbed tables (random geometry, 10 nonzero TRiSK
    weights, shortened edges-on-edge lists, random del2/del4 scaling; with
    `full` also a 0/1 edge mask on 20 % of the edge levels and dv < dc/4 on
    5 % of the edges, where the del4 chain's first Laplacian uses
    1/max(dv, dc/4)): tendency and 5-step trajectory dot products against
    the tangent-linear model <= 1e-12; tables that no consistent mesh has
    are rejected."""
    cut = general_mesh(10, 8, 4, 7373, adjoint_ready=True, cut_cells=True)
    with pytest.raises(og.SwgError, match="neighbour"):
        og.Adjoint(models(*cut, 2)[2], 2)
    om, gm = general_mesh(10, 8, 4, 7373, adjoint_ready=not full,
                          cut_cells=False)
    if full:
        assert not np.all(om.tables["edge_mask"] == 1.0)
        assert np.any(om.tables["dv_edge"] < 0.25 * om.tables["dc_edge"])
    T = 2
    _, gp, model = models(om, gm, T)
    adj = og.Adjoint(model, 2, stepper, nstages)
    x = state(om, T, 41)
    C_, E, K = om.ncells, om.nedges, om.nlayers
    dx = (uniform(51, C_ * K).reshape(C_, K) - 0.5,
          0.01 * (uniform(52, E * K).reshape(E, K) - 0.5),
          10 * (uniform(53, T * C_ * K).reshape(T, C_, K) - 0.5))
    mu = tuple(uniform(61 + j, a.size).reshape(a.shape) - 0.5
               for j, a in enumerate(x))

    def mk(a):
        st = og.ShallowWaterState(gm, gp)
        st.upload(*a)
        return st

    def dot(a, b):
        return sum(float(np.sum(p * q)) for p, q in zip(a, b))

    X = mk(x)
    JD, JT = og.ShallowWaterState(gm, gp), og.ShallowWaterState(gm, gp)
    adj.tlm_tendency(X, mk(dx), JD)
    adj.adj_tendency(X, mk(mu), JT)
    lhs, rhs = dot(JD.download(), mu), dot(dx, JT.download())
    assert abs(lhs - rhs) <= TOL * max(abs(lhs), abs(rhs)), (lhs, rhs)
    XN = og.ShallowWaterState(gm, gp)
    adj.forward(X, 0.0, 5.0, 5, XN)
    LAM = mk(mu)
    adj.backward(LAM)
    DX = mk(dx)
    adj.tlm_apply(X, DX, 0.0, 5.0, 5)
    lhs, rhs = dot(DX.download(), mu), dot(dx, LAM.download())
    assert abs(lhs - rhs) <= TOL * max(abs(lhs), abs(rhs)), (lhs, rhs)


@pytest.mark.parametrize("scale2", [1.0, 0.37])
def test_uniform_del2_scaling_folds_tracer_del2(scale2):
    """mesh_scaling_del2 equal on every edge: the tracer del2 term is
    eddy_diff2 * s times the del4 term's thickness-weighted Laplacian and
    enters through the centre weight of the del4 stencil.  Against the
    oracle (which sums the reference's del2 weights): tendency and 3 LSRK5
    steps <= 1e-12, also with tracer del4 switched off at run time (the
    separate del2 weights again) and through the no-allocation entry point."""
    om, gm0 = general_mesh(10, 8, 7, 6262, adjoint_ready=True)
    t = om.tables
    t["mesh_scaling_del2"][:] = scale2
    gm = og.MPASMesh.from_tables(
        {n: t[n] for n in TABLES}, 7,
        mesh_scaling_del2=t["mesh_scaling_del2"],
        mesh_scaling_del4=t["mesh_scaling_del4"], edge_mask=t["edge_mask"],
        max_level_cell=om.max_level_cell,
        max_level_vertex_bot=om.max_level_vertex_bot)
    T = 3
    omd, gp, model = models(om, gm, T)
    x = state(om, T, 515)
    want = omd.compute_tendency(*x, t=0.0)
    S = og.ShallowWaterState(gm, gp)
    S.upload(*x)
    Tn = og.ShallowWaterState(gm, gp)
    model.compute_tendency(Tn, S, 0.0)
    for got, ref in zip(Tn.download(), want):
        assert rel_diff(got, ref) <= TOL
    # no-allocation entry point, same tables and parameters
    from test_zz_no_alloc import _noalloc
    Tz = og.ShallowWaterState(gm, gp)
    assert _noalloc(gm, gp, S, Tz, 0) == 0
    for got, ref in zip(Tz.download(), want):
        assert rel_diff(got, ref) <= TOL
    want = omd.step(*(a.copy() for a in x), 0.0, 5.0, 3, kind="lsrk",
                    nstages=5)
    st = og.LSRKStepper(model, 5)
    st.step(S, 0.0, 5.0, 3)
    for got, ref in zip(S.download(), want):
        assert rel_diff(got, ref) <= TOL
    # tracer del4 off: del2 through its own weights again
    model.m_tracer_hyperdiff_cell.m_enabled = False
    omd.set_term(8, False)
    S.upload(*x)
    model.compute_tendency(Tn, S, 0.0)
    want = omd.compute_tendency(*x, t=0.0)
    for got, ref in zip(Tn.download(), want):
        assert rel_diff(got, ref) <= TOL
