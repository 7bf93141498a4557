"""Gradient with respect to a per-cell del2 viscosity field (realised through
mesh_scaling_del2), checked by central finite differences, and batched
ensemble adjoints (uneven members, different checkpoint budgets, one stream
each) checked bitwise against each member's own adjoint."""
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


def check_batched_adjoint(wls, budgets):
    """Batched adjoints (one stream per member) bitwise equal to each
    member's own adjoint run alone: gradients w.r.t. the initial state and
    the per-cell viscosity."""
    torch = pytest.importorskip("torch")
    members = []
    for i, wl in enumerate(wls):
        visc = lognormal_visc(wl.nx * wl.ny, wl.seed + 5)
        mesh, params, model = build(wl, visc)
        members.append((wl, mesh, params, model, initial_state(mesh, wl),
                        region_cells(mesh, wl.seed + 99), budgets[i]))

    def one(m):
        wl, mesh, params, model, x0, region, budget = m
        adj = og.Adjoint(model, budget)
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
        ref.append((G.download(), adj.grad_visc()[1]))
        del adj, X0, XN, G
    # all members together, one stream each
    objs = [one(m) for m in members]
    streams = [torch.cuda.Stream() for _ in members]
    og.adjoint_batch_forward([o[0] for o in objs], [o[1] for o in objs], 0.0,
                             wls[0].dt, wls[0].nsteps, [o[2] for o in objs],
                             [s.cuda_stream for s in streams])
    torch.cuda.synchronize()
    Gs = []
    for o, m in zip(objs, members):
        _, g = loss_and_grad(*o[2].download(), m[5])
        G = og.ShallowWaterState(m[1], m[2])
        G.upload(*g)
        Gs.append(G)
    og.adjoint_batch_backward([o[0] for o in objs], Gs,
                              [s.cuda_stream for s in streams])
    torch.cuda.synchronize()
    for i, (G, o) in enumerate(zip(Gs, objs)):
        for a, b in zip(G.download(), ref[i][0]):
            np.testing.assert_array_equal(a, b, err_msg=f"member {i}")
        np.testing.assert_array_equal(o[0].grad_visc()[1], ref[i][1])


def test_batched_adjoint_equals_single_member_adjoints():
    """6 uneven members, budgets 2 to 21 snapshots, 20 steps."""
    wls = adjoint_ensemble(n=6, nx_choices=(8, 12, 16), levels=(4, 12),
                           nsteps=20)
    check_batched_adjoint(wls, [2, 3, 4, 5, 6, 21])


def test_batched_adjoint_full_ensemble_workload():
    """The full 32-member ensemble: nx in {32, 64, 96, 128}, 16-64 levels,
    2 tracers, RK4, 300 steps, 32 snapshots (16 for nx = 128)."""
    wls = adjoint_ensemble(n=32)
    check_batched_adjoint(wls, [16 if wl.nx >= 128 else 32 for wl in wls])


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
