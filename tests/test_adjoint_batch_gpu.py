"""Gradient with respect to a per-cell del2 viscosity field (realised through
mesh_scaling_del2), checked by central finite differences, and ensemble
adjoints (uneven members, different checkpoint budgets) checked bitwise
against each member's own adjoint: the batched ensemble (swg_adj_ensemble_*,
one launch per pass over the members of a lockstep group) and the
stream-interleaved form (swg_adj_batch_*, one stream per member)."""
import numpy as np
import pytest

import omega_playground_gb300 as og
from omega_playground_gb300.workloads import (adjoint_ensemble, initial_state,
                                              lognormal_visc, loss_and_grad,
                                              region_cells, uniform,
                                              visc_scaling)

pytestmark = pytest.mark.gpu


def build(wl, visc_cell):
    probe = og.PlanarHexagonalMesh(wl.nx, wl.ny, wl.dc, wl.nlayers)
    scale = visc_scaling(probe, visc_cell, wl.visc_del2)
    mesh = og.PlanarHexagonalMesh(wl.nx, wl.ny, wl.dc, wl.nlayers,
                                  mesh_scaling_del2=scale)
    params = wl.params()
    return mesh, params, og.ShallowWaterModel(mesh, params)


def run_loss(wl, visc_cell, x0, region, nsteps):
    mesh, params, model = build(wl, visc_cell)
    s = og.ShallowWaterState(mesh, params)
    s.upload(*x0)
    og.RK4Stepper(model).step(s, 0.0, wl.dt, nsteps)
    return loss_and_grad(*s.download(), region)[0]


def test_viscosity_field_gradient_fd():
    wl = adjoint_ensemble(n=1, nx_choices=(16,), levels=(6, 6), nsteps=40)[0]
    visc = lognormal_visc(wl.nx * wl.ny, wl.seed + 5)
    mesh, params, model = build(wl, visc)
    region = region_cells(mesh, wl.seed + 99)
    x0 = initial_state(mesh, wl)
    adj = og.Adjoint(model, 5)
    with pytest.raises(og.SwgError, match="no backward sweep"):
        adj.grad_visc()                      # nothing to report yet
    X0 = og.ShallowWaterState(mesh, params)
    X0.upload(*x0)
    XN = og.ShallowWaterState(mesh, params)
    adj.forward(X0, 0.0, wl.dt, wl.nsteps, XN)
    _, g = loss_and_grad(*XN.download(), region)
    G = og.ShallowWaterState(mesh, params)
    G.upload(*g)
    adj.backward(G)
    _, gcell = adj.grad_visc()
    # The directions are positive random weights per cell (0.5 to 1.5 times
    # the local viscosity): with random signs the directional derivative is
    # about 1e-6 of the loss, and the rounding of the loss (h near 1000 m,
    # about 1e-11 absolute) would then dominate the central difference.
    # Central differences at eps and eps/2 are combined by Richardson
    # extrapolation so that their O(eps^2) truncation term cancels.
    eps = 1e-3  # relative perturbation of the field

    def central(d, e):
        lp = run_loss(wl, visc + e * d, x0, region, wl.nsteps)
        lm = run_loss(wl, visc - e * d, x0, region, wl.nsteps)
        return (lp - lm) / (2 * e)

    for j in range(4):
        u = uniform(700 + j, visc.size)
        d = (0.5 + u) * visc          # relative direction
        f1 = central(d, eps)
        f2 = central(d, eps / 2)
        fd = (4 * f2 - f1) / 3
        an = float(np.dot(gcell, d))
        assert abs(fd - an) <= 1e-6 * abs(an), (j, f1, f2, fd, an)


def check_batched_adjoint(wls, budgets, ensemble=False, kind="rk4",
                          nstages=4, switch=None):
    """Ensemble adjoints bitwise equal to each member's own adjoint run
    alone: gradients w.r.t. the initial state and the per-cell viscosity,
    x_N, and the schedule counts.  ensemble: swg_adj_ensemble_* (batched
    launches per lockstep group); else swg_adj_batch_* (one stream per
    member).  switch: a term switched off on every member's model."""
    torch = pytest.importorskip("torch")
    members = []
    for i, wl in enumerate(wls):
        visc = lognormal_visc(wl.nx * wl.ny, wl.seed + 5)
        mesh, params, model = build(wl, visc)
        if switch:
            getattr(model, switch).m_enabled = False
        members.append((wl, mesh, params, model, initial_state(mesh, wl),
                        region_cells(mesh, wl.seed + 99), budgets[i]))

    def one(m):
        wl, mesh, params, model, x0, region, budget = m
        adj = og.Adjoint(model, budget, kind, nstages)
        X0 = og.ShallowWaterState(mesh, params)
        X0.upload(*x0)
        XN = og.ShallowWaterState(mesh, params)
        return adj, X0, XN

    # single members, one after the other
    ref = []
    for m in members:
        adj, X0, XN = one(m)
        adj.forward(X0, 0.0, m[0].dt, m[0].nsteps, XN)
        _, g = loss_and_grad(*XN.download(), m[5])
        G = og.ShallowWaterState(m[1], m[2])
        G.upload(*g)
        adj.backward(G)
        ref.append((G.download(), adj.grad_visc()[1], XN.download(),
                    adj.info_ex()))
        del adj, X0, XN, G
    objs = [one(m) for m in members]
    if ensemble:  # batched launches per lockstep group
        ens = og.AdjointEnsemble([o[0] for o in objs])
        ens.forward([o[1] for o in objs], 0.0, wls[0].dt, wls[0].nsteps,
                    [o[2] for o in objs])
    else:  # one stream each
        streams = [torch.cuda.Stream() for _ in members]
        og.adjoint_batch_forward([o[0] for o in objs], [o[1] for o in objs],
                                 0.0, wls[0].dt, wls[0].nsteps,
                                 [o[2] for o in objs],
                                 [s.cuda_stream for s in streams])
    torch.cuda.synchronize()
    Gs = []
    for o, m in zip(objs, members):
        _, g = loss_and_grad(*o[2].download(), m[5])
        G = og.ShallowWaterState(m[1], m[2])
        G.upload(*g)
        Gs.append(G)
    if ensemble:
        ens.backward(Gs)
    else:
        og.adjoint_batch_backward([o[0] for o in objs], Gs,
                                  [s.cuda_stream for s in streams])
    torch.cuda.synchronize()
    for i, (G, o) in enumerate(zip(Gs, objs)):
        for a, b in zip(G.download(), ref[i][0]):
            np.testing.assert_array_equal(a, b, err_msg=f"member {i}")
        for a, b in zip(o[2].download(), ref[i][2]):
            np.testing.assert_array_equal(a, b, err_msg=f"member {i} x_N")
        np.testing.assert_array_equal(o[0].grad_visc()[1], ref[i][1])
        assert o[0].info_ex() == ref[i][3]
    return ens if ensemble else None


@pytest.mark.parametrize("ensemble", [False, True])
def test_batched_adjoint_equals_single_member_adjoints(ensemble):
    """6 uneven members, budgets 2 to 21 snapshots, 20 steps; in the
    ensemble, budgets 2 and 3 are shared by two members each (groups of
    two), the rest run alone."""
    wls = adjoint_ensemble(n=6, nx_choices=(8, 12, 16), levels=(4, 12),
                           nsteps=20)
    budgets = [2, 3, 2, 3, 6, 21] if ensemble else [2, 3, 4, 5, 6, 21]
    ens = check_batched_adjoint(wls, budgets, ensemble)
    if ensemble:
        assert ens.groups() == (4, [0, 1, 0, 1, 2, 3])


@pytest.mark.parametrize("ensemble", [False, True])
def test_batched_adjoint_full_ensemble_workload(ensemble):
    """The full 32-member ensemble: nx in {32, 64, 96, 128}, 16-64 levels,
    2 tracers, RK4, 300 steps, 32 snapshots (16 for nx = 128); batched, it
    runs as two lockstep groups (the two budgets)."""
    wls = adjoint_ensemble(n=32)
    ens = check_batched_adjoint(wls, [16 if wl.nx >= 128 else 32
                                      for wl in wls], ensemble)
    if ensemble:
        assert ens.groups()[0] == 2


@pytest.mark.parametrize("kind,nstages", [("lsrk", 5), ("lsrk", 1)])
def test_ensemble_low_storage_steppers(kind, nstages):
    """The batched ensemble with the 5-stage and 1-stage low-storage steppers
    (odd stage counts: the step's first mu is formed per step)."""
    wls = adjoint_ensemble(n=4, nx_choices=(8, 12), levels=(3, 6), nsteps=9)
    check_batched_adjoint(wls, [2, 2, 3, 3], True, kind, nstages)


@pytest.mark.parametrize("switch", ["m_pv_flux_edge", "m_ssh_grad_edge",
                                    "m_tracer_hadv_cell"])
def test_ensemble_with_a_switched_term(switch):
    wls = adjoint_ensemble(n=3, nx_choices=(8, 12), levels=(3, 6), nsteps=7)
    check_batched_adjoint(wls, [2, 2, 2], True, switch=switch)


def test_batched_adjoint_rejects_members_sharing_a_model():
    wl = adjoint_ensemble(n=1, nx_choices=(8,), levels=(4, 4), nsteps=4)[0]
    mesh, params, model = build(wl, lognormal_visc(wl.nx * wl.ny, 3))
    adjs = [og.Adjoint(model, 2), og.Adjoint(model, 2)]
    x0 = initial_state(mesh, wl)
    X = [og.ShallowWaterState(mesh, params) for _ in range(4)]
    for s in X[:2]:
        s.upload(*x0)
    with pytest.raises(og.SwgError):
        og.adjoint_batch_forward(adjs, X[:2], 0.0, wl.dt, 4, X[2:])


def test_ensemble_rejects_members_sharing_a_model_and_a_stale_backward():
    wl = adjoint_ensemble(n=1, nx_choices=(8,), levels=(4, 4), nsteps=4)[0]
    mesh, params, model = build(wl, lognormal_visc(wl.nx * wl.ny, 3))
    with pytest.raises(og.SwgError):
        og.AdjointEnsemble([og.Adjoint(model, 2), og.Adjoint(model, 2)])
    adj = og.Adjoint(model, 2)
    ens = og.AdjointEnsemble([adj])
    X = [og.ShallowWaterState(mesh, params) for _ in range(2)]
    X[0].upload(*initial_state(mesh, wl))
    with pytest.raises(og.SwgError):
        ens.backward([X[1]])                 # no forward sweep yet
    ens.forward([X[0]], 0.0, wl.dt, 4, [X[1]])
    model.m_ke_grad_edge.m_enabled = False
    with pytest.raises(og.SwgError, match="switched"):
        ens.backward([X[1]])
    model.m_ke_grad_edge.m_enabled = True
    ens.backward([X[1]])
