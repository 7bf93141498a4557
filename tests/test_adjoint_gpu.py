"""Tangent-linear and adjoint models.

- dot-product tests: <J dx, mu> = <dx, J^T mu> for one tendency evaluation
  (every term on, and the frozen-flow tracer configuration), and
  <dx_N, lam_N> = <dx_0, lam_0> over RK4 trajectories whose adjoint runs
  through the binomial checkpointing schedule (several snapshot budgets);
  bound 1e-12 relative.  The TLM is the forward kernels on dual numbers, the
  adjoint is hand-written, so agreement checks the adjoint;
- central finite differences of the plain forward (16 seeded directions)
  against the adjoint gradient of the region loss; bound 1e-6 relative."""
import numpy as np
import pytest

import omega_playground_gb300 as og
from omega_playground_gb300.workloads import (WORKLOADS, initial_state,
                                              loss_and_grad, region_cells,
                                              uniform)

pytestmark = pytest.mark.gpu


def setup(wl, **over):
    mesh = og.PlanarHexagonalMesh(wl.nx, wl.ny, wl.dc, wl.nlayers)
    params = wl.params()
    for k, v in over.items():
        setattr(params, k, v)
    model = og.ShallowWaterModel(mesh, params)
    return mesh, params, model


def rand_like(shapes, seed, scale=(1.0, 1.0, 1.0)):
    out = []
    for j, (sh, sc) in enumerate(zip(shapes, scale)):
        n = int(np.prod(sh))
        u = uniform(seed + 7 * j, 2 * n)
        g = np.sqrt(-2 * np.log(u[:n] + 1e-300)) * np.cos(2 * np.pi * u[n:])
        out.append(sc * g.reshape(sh))
    return out


def dot(a, b):
    return sum(float(np.sum(x * y)) for x, y in zip(a, b))


def make_state(mesh, params, arrays):
    s = og.ShallowWaterState(mesh, params)
    s.upload(*arrays)
    return s


ALL_TERMS = WORKLOADS["lsrk5_512x512"].scaled(nx=12, ny=10, nlayers=5,
                                              ntracers=3, stepper="rk4",
                                              nstages=4)


@pytest.mark.parametrize("over", [{}, {"m_disable_h_tendency": True,
                                       "m_disable_vn_tendency": True},
                                  {"m_disable_h_tendency": True},
                                  {"m_disable_vn_tendency": True},
                                  {"m_visc_del4": 0.0, "m_eddy_diff4": 0.0}])
def test_tendency_dot_product(over):
    mesh, params, model = setup(ALL_TERMS, **over)
    adj = og.Adjoint(model, 2)
    x = initial_state(mesh, ALL_TERMS)
    shapes = [a.shape for a in x]
    dx = rand_like(shapes, 101, (1.0, 0.01, 10.0))
    mu = rand_like(shapes, 202)
    X = make_state(mesh, params, x)
    DX = make_state(mesh, params, dx)
    MU = make_state(mesh, params, mu)
    JT = og.ShallowWaterState(mesh, params)
    JD = og.ShallowWaterState(mesh, params)
    adj.tlm_tendency(X, DX, JD)
    adj.adj_tendency(X, MU, JT)
    jd, jt = JD.download(), JT.download()
    lhs, rhs = dot(jd, mu), dot(dx, jt)
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs)), (lhs, rhs)
    # the TLM against a central difference of the forward tendency
    eps = 1e-6
    tp = og.ShallowWaterState(mesh, params)
    tm = og.ShallowWaterState(mesh, params)
    model.compute_tendency(tp, make_state(mesh, params,
                                          [a + eps * b for a, b in zip(x, dx)]), 0.0)
    model.compute_tendency(tm, make_state(mesh, params,
                                          [a - eps * b for a, b in zip(x, dx)]), 0.0)
    fd = [(p - q) / (2 * eps) for p, q in zip(tp.download(), tm.download())]
    for a, b in zip(fd, jd):
        scale = max(np.max(np.abs(b)), 1e-300)
        assert np.max(np.abs(a - b)) / scale < 1e-5


@pytest.mark.parametrize("nsteps,nsnap,over", [
    (1, 1, {}), (7, 1, {}), (7, 3, {}), (20, 4, {}), (9, 12, {}),
    (6, 2, {"m_disable_h_tendency": True}),
    (6, 2, {"m_disable_vn_tendency": True})])
def test_trajectory_dot_product_through_checkpointing(nsteps, nsnap, over):
    """RK4 adjoint against the tangent-linear model through schedules of 1
    to 12 snapshots, <= 1e-12, and the forward sweep's x_N bitwise equal to
    the plain stepper's; also with h or vn frozen (a frozen field of x_N is
    the step's input, which the taped last step copies)."""
    wl = ALL_TERMS
    mesh, params, model = setup(wl, **over)
    adj = og.Adjoint(model, nsnap)
    x0 = initial_state(mesh, wl)
    shapes = [a.shape for a in x0]
    dx0 = rand_like(shapes, 303, (1.0, 0.01, 10.0))
    lamN = rand_like(shapes, 404)
    X0 = make_state(mesh, params, x0)
    XN = og.ShallowWaterState(mesh, params)
    adj.forward(X0, 0.0, wl.dt, nsteps, XN)
    LAM = make_state(mesh, params, lamN)
    adj.backward(LAM)
    lam0 = LAM.download()
    plain, taped, tadv = adj.info_ex()
    assert taped == nsteps
    assert (plain, tadv) == og.adjoint_plan(nsteps, nsnap, 4)
    DX = make_state(mesh, params, dx0)
    adj.tlm_apply(X0, DX, 0.0, wl.dt, nsteps)
    dxN = DX.download()
    lhs, rhs = dot(dxN, lamN), dot(dx0, lam0)
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs)), (lhs, rhs)
    # the forward sweep's final state equals a plain RK4 run
    ref = make_state(mesh, params, x0)
    og.RK4Stepper(model).step(ref, 0.0, wl.dt, nsteps, use_graph=False)
    for a, b in zip(XN.download(), ref.download()):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("nx,ny", [(1, 1), (1, 2), (2, 3)])
@pytest.mark.parametrize("stepper,nstages", [("rk4", 4), ("lsrk", 5)])
def test_tiny_mesh_dot_products(nx, ny, stepper, nstages):
    """The smallest meshes, where a cell is its own neighbour and an edge
    appears several times in another's edges-on-edge list (the transposed
    tables then hold repeated entries): tendency and 6-step trajectory dot
    products <= 1e-12."""
    wl = ALL_TERMS.scaled(nx=nx, ny=ny, nlayers=3, ntracers=2)
    mesh, params, model = setup(wl)
    adj = og.Adjoint(model, 2, stepper, nstages)
    x0 = initial_state(mesh, wl)
    shapes = [a.shape for a in x0]
    dx, mu = rand_like(shapes, 505, (1.0, 0.01, 10.0)), rand_like(shapes, 606)
    X = make_state(mesh, params, x0)
    JD, JT = og.ShallowWaterState(mesh, params), og.ShallowWaterState(mesh, params)
    adj.tlm_tendency(X, make_state(mesh, params, dx), JD)
    adj.adj_tendency(X, make_state(mesh, params, mu), JT)
    lhs, rhs = dot(JD.download(), mu), dot(dx, JT.download())
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs)), (lhs, rhs)
    XN = og.ShallowWaterState(mesh, params)
    adj.forward(X, 0.0, wl.dt, 6, XN)
    LAM = make_state(mesh, params, mu)
    adj.backward(LAM)
    DX = make_state(mesh, params, dx)
    adj.tlm_apply(X, DX, 0.0, wl.dt, 6)
    lhs, rhs = dot(DX.download(), mu), dot(dx, LAM.download())
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs)), (lhs, rhs)


def _fd_check(wl, nsteps, nsnap, ndir, eps, stepper="rk4", nstages=4,
              richardson=False):
    """Worst relative difference between the adjoint gradient and central
    differences over ndir seeded directions; with richardson the central
    differences at eps and eps/2 are combined so that their O(eps^2)
    truncation term cancels."""
    mesh, params, model = setup(wl)
    region = region_cells(mesh, wl.seed + 99)
    assert len(region) > 0
    x0 = initial_state(mesh, wl)
    adj = og.Adjoint(model, nsnap, stepper, nstages)
    X0 = make_state(mesh, params, x0)
    XN = og.ShallowWaterState(mesh, params)
    adj.forward(X0, 0.0, wl.dt, nsteps, XN)
    L0, g = loss_and_grad(*XN.download(), region)
    G = make_state(mesh, params, g)
    adj.backward(G)
    grad = G.download()
    stepper = (og.RK4Stepper(model) if stepper == "rk4"
               else og.LSRKStepper(model, nstages))
    shapes = [a.shape for a in x0]
    worst = 0.0
    for j in range(ndir):
        d = rand_like(shapes, 1000 + 17 * j, (1.0, 0.01, 10.0))
        def central(e):
            vals = []
            for sgn in (1, -1):
                s = make_state(mesh, params,
                               [a + sgn * e * b for a, b in zip(x0, d)])
                stepper.step(s, 0.0, wl.dt, nsteps)
                vals.append(loss_and_grad(*s.download(), region)[0])
            return (vals[0] - vals[1]) / (2 * e)
        fd = central(eps)
        if richardson:
            fd = (4 * central(eps / 2) - fd) / 3
        an = dot(grad, d)
        worst = max(worst, abs(fd - an) / abs(an))
    return worst


def test_finite_differences_reduced():
    """The adjoint workload's physics on a 32x32x8 mesh, 60 RK4 steps, 6
    snapshots, 16 seeded directions."""
    wl = WORKLOADS["rk4_128x128_adjoint"].scaled(nx=32, ny=32, nlayers=8)
    assert _fd_check(wl, 60, 6, 16, 1e-4) <= 1e-6


def test_finite_differences_full_adjoint_workload():
    """128x128 cells, 32 levels, 2 tracers, RK4, 1000 steps, 32 snapshots,
    16 seeded directions."""
    wl = WORKLOADS["rk4_128x128_adjoint"]
    assert _fd_check(wl, wl.nsteps, 32, 16, 1e-4) <= 1e-6


def test_dot_product_full_adjoint_workload():
    """The adjoint workload itself (128x128 cells, 32 levels, 2 tracers,
    RK4, 1000 steps, 32 snapshots): <dx_N, lam_N> from the tangent-linear
    model against <dx_0, lam_0> from the checkpointed adjoint, <= 1e-12."""
    wl = WORKLOADS["rk4_128x128_adjoint"]
    mesh, params, model = setup(wl)
    adj = og.Adjoint(model, 32)
    x0 = initial_state(mesh, wl)
    shapes = [a.shape for a in x0]
    dx0 = rand_like(shapes, 515, (1.0, 0.01, 10.0))
    lamN = rand_like(shapes, 616)
    X0 = make_state(mesh, params, x0)
    XN = og.ShallowWaterState(mesh, params)
    adj.forward(X0, 0.0, wl.dt, wl.nsteps, XN)
    LAM = make_state(mesh, params, lamN)
    adj.backward(LAM)
    plain, tadv = og.adjoint_plan(wl.nsteps, 32, 4)
    assert adj.info_ex() == (plain, wl.nsteps, tadv)
    assert plain + tadv < og.checkpoint_cost(wl.nsteps, 32)
    DX = make_state(mesh, params, dx0)
    adj.tlm_apply(X0, DX, 0.0, wl.dt, wl.nsteps)
    lhs, rhs = dot(DX.download(), lamN), dot(dx0, LAM.download())
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs)), \
        (lhs, rhs, abs(lhs - rhs) / max(abs(lhs), abs(rhs)))


def test_checkpoint_budget_and_step_limit_are_errors():
    """A budget whose schedule would re-run more than 32 plain steps per step
    is SWG_ERR_BUDGET (one snapshot for 200 steps: 99.5 per step); more steps
    than the planner takes is SWG_ERR_ARG; both leave the adjoint usable."""
    wl = ALL_TERMS
    mesh, params, model = setup(wl)
    adj = og.Adjoint(model, 1)
    x0 = initial_state(mesh, wl)
    X0 = make_state(mesh, params, x0)
    XN = og.ShallowWaterState(mesh, params)
    with pytest.raises(og.SwgError) as e:
        adj.forward(X0, 0.0, wl.dt, 200, XN)
    assert e.value.code == 5
    with pytest.raises(og.SwgError) as e:
        og.Adjoint(model, 32).forward(X0, 0.0, wl.dt, 10001, XN)
    assert e.value.code == 1
    adj.forward(X0, 0.0, wl.dt, 20, XN)   # 90 plain steps: within budget
    LAM = make_state(mesh, params, rand_like([a.shape for a in x0], 5))
    adj.backward(LAM)
    assert adj.info_ex() == (90, 20, 11) and og.adjoint_plan(20, 1) == (90, 11)


@pytest.mark.parametrize("nstages,nsteps,nsnap,over", [
    (5, 1, 1, {}), (5, 7, 3, {}), (5, 20, 4, {}), (1, 9, 2, {}),
    (1, 12, 12, {}), (5, 6, 2, {"m_disable_h_tendency": True}),
    (5, 6, 2, {"m_disable_vn_tendency": True})])
def test_lsrk_trajectory_dot_product_through_checkpointing(nstages, nsteps,
                                                           nsnap, over):
    """The low-storage RK adjoint (5-stage Carpenter-Kennedy and 1-stage
    Euler) against its dual-number tangent-linear model, <= 1e-12, and the
    forward sweep's x_N bitwise equal to the plain LSRK stepper's; also with
    h or vn frozen."""
    wl = ALL_TERMS
    mesh, params, model = setup(wl, **over)
    adj = og.Adjoint(model, nsnap, "lsrk", nstages)
    x0 = initial_state(mesh, wl)
    shapes = [a.shape for a in x0]
    dx0 = rand_like(shapes, 313, (1.0, 0.01, 10.0))
    lamN = rand_like(shapes, 414)
    X0 = make_state(mesh, params, x0)
    XN = og.ShallowWaterState(mesh, params)
    adj.forward(X0, 0.0, wl.dt, nsteps, XN)
    LAM = make_state(mesh, params, lamN)
    adj.backward(LAM)
    lam0 = LAM.download()
    plain, taped, tadv = adj.info_ex()
    assert taped == nsteps
    assert (plain, tadv) == og.adjoint_plan(nsteps, nsnap, nstages)
    DX = make_state(mesh, params, dx0)
    adj.tlm_apply(X0, DX, 0.0, wl.dt, nsteps)
    lhs, rhs = dot(DX.download(), lamN), dot(dx0, lam0)
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs)), (lhs, rhs)
    ref = make_state(mesh, params, x0)
    og.LSRKStepper(model, nstages).step(ref, 0.0, wl.dt, nsteps,
                                        use_graph=False)
    for a, b in zip(XN.download(), ref.download()):
        np.testing.assert_array_equal(a, b)


def test_lsrk5_finite_differences_reduced():
    """The LSRK5 adjoint of the region loss against central differences of
    the plain LSRK5 forward: 32x32x8, 60 steps, 6 snapshots, 16 seeded
    directions, Richardson-extrapolated central differences at eps = 1e-3
    and 5e-4, <= 1e-6.  (A plain central difference at eps = 1e-4 reached
    1.1e-6 in its worst direction: the difference's own error, not the
    adjoint's, which the dot-product test bounds at 1e-12.)"""
    wl = WORKLOADS["rk4_128x128_adjoint"].scaled(nx=32, ny=32, nlayers=8)
    assert _fd_check(wl, 60, 6, 16, 1e-3, "lsrk", 5, richardson=True) <= 1e-6
