"""PyTorch autograd over the derivative entry points
(omega_playground_gb300/autograd.py).

- the Functions' vjp / jvp equal the direct swg_adj_* / swg_tlm_* calls bit
  for bit (same kernels, same stream), for the tendency and for RK4 and LSRK5
  rollouts through the binomial checkpointing schedule;
- dot-product tests through torch alone: <J dx, mu> from forward-mode AD
  against <dx, J^T mu> from torch.autograd.grad, bound 1e-12 relative;
- a rollout graph whose checkpoints were overwritten by a later rollout
  raises instead of returning another trajectory's gradient."""
import numpy as np
import pytest

import omega_playground_gb300 as og
from omega_playground_gb300.workloads import WORKLOADS, initial_state, uniform

torch = pytest.importorskip("torch")
from omega_playground_gb300 import autograd as oga  # noqa: E402
from torch.autograd import forward_ad  # noqa: E402

pytestmark = pytest.mark.gpu

WL = WORKLOADS["lsrk5_512x512"].scaled(nx=12, ny=10, nlayers=5, ntracers=2,
                                       stepper="rk4", nstages=4)
DT, NSTEPS = 20.0, 12


def setup(stepper="rk4", nstages=4, nsnap=3):
    mesh = og.PlanarHexagonalMesh(WL.nx, WL.ny, WL.dc, WL.nlayers)
    params = WL.params()
    model = og.ShallowWaterModel(mesh, params)
    adj = og.Adjoint(model, nsnap, stepper=stepper, nstages=nstages)
    x = [torch.from_numpy(a.copy()).cuda() for a in initial_state(mesh, WL)]
    return mesh, params, model, adj, x


def rand_like(x, seed, scale=(1.0, 0.01, 10.0)):
    return [torch.from_numpy(s * (uniform(seed + j, t.numel()) - 0.5)
                             .reshape(tuple(t.shape))).cuda()
            for j, (t, s) in enumerate(zip(x, scale))]


def dot(a, b):
    return sum(float((u * v).sum()) for u, v in zip(a, b))


def state(mesh, params, fields):
    s = og.ShallowWaterState(mesh, params)
    s.upload(*[t.cpu().numpy() for t in fields])
    return s


def test_tendency_matches_direct_calls_and_dot_product():
    mesh, params, model, adj, x = setup()
    dx, mu = rand_like(x, 11), rand_like(x, 23, (1.0, 1.0, 1.0))
    xs = [t.clone().requires_grad_(True) for t in x]
    f = oga.tendency(adj, *xs)
    lam = torch.autograd.grad(f, xs, grad_outputs=mu)
    with forward_ad.dual_level():
        duals = [forward_ad.make_dual(t, d) for t, d in zip(x, dx)]
        jd = [forward_ad.unpack_dual(o).tangent
              for o in oga.tendency(adj, *duals)]
    # direct calls on the same inputs
    X, DX, MU = (state(mesh, params, v) for v in (x, dx, mu))
    T, JD, LAM = (og.ShallowWaterState(mesh, params) for _ in range(3))
    model.compute_tendency(T, X, 0.0)
    adj.tlm_tendency(X, DX, JD)
    adj.adj_tendency(X, MU, LAM)
    for got, want in ((f, T), (jd, JD), (lam, LAM)):
        for g, w in zip(got, want.download()):
            np.testing.assert_array_equal(g.detach().cpu().numpy(), w)
    lhs, rhs = dot(jd, mu), dot(dx, lam)
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs)), (lhs, rhs)


@pytest.mark.parametrize("stepper,nstages", [("rk4", 4), ("lsrk", 5)])
def test_rollout_matches_direct_calls_and_dot_product(stepper, nstages):
    mesh, params, model, adj, x = setup(stepper, nstages)
    dx, w = rand_like(x, 31), rand_like(x, 47, (1.0, 1.0, 1.0))
    xs = [t.clone().requires_grad_(True) for t in x]
    xn = oga.rollout(adj, *xs, 0.0, DT, NSTEPS)
    loss = sum((a * b).sum() for a, b in zip(xn, w))
    grad = torch.autograd.grad(loss, xs)
    with forward_ad.dual_level():
        duals = [forward_ad.make_dual(t, d) for t, d in zip(x, dx)]
        dxn = [forward_ad.unpack_dual(o).tangent
               for o in oga.rollout(adj, *duals, 0.0, DT, NSTEPS)]
    # direct calls through a second adjoint with the same budget
    ref = og.Adjoint(model, 3, stepper=stepper, nstages=nstages)
    X0, XN = state(mesh, params, x), og.ShallowWaterState(mesh, params)
    ref.forward(X0, 0.0, DT, NSTEPS, XN)
    LAM = state(mesh, params, w)
    ref.backward(LAM)
    DX = state(mesh, params, dx)
    ref.tlm_apply(state(mesh, params, x), DX, 0.0, DT, NSTEPS)
    for got, want in ((xn, XN), (grad, LAM), (dxn, DX)):
        for g, v in zip(got, want.download()):
            np.testing.assert_array_equal(g.detach().cpu().numpy(), v)
    lhs, rhs = dot(dxn, w), dot(dx, grad)
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs)), (lhs, rhs)


def test_overwritten_checkpoints_raise():
    _, _, _, adj, x = setup()
    xs = [t.clone().requires_grad_(True) for t in x]
    first = oga.rollout(adj, *xs, 0.0, DT, 4)
    second = oga.rollout(adj, *xs, 0.0, DT, 5)
    with pytest.raises(RuntimeError, match="checkpoints"):
        torch.autograd.grad(first[0].sum(), xs)
    torch.autograd.grad(second[0].sum(), xs)       # the live one works
    third = oga.rollout(adj, *xs, 0.0, DT, 4)
    torch.autograd.grad(third[0].sum(), xs, retain_graph=True)
    with pytest.raises(RuntimeError, match="checkpoints"):
        torch.autograd.grad(third[0].sum(), xs)    # consumed by the first backward


def test_inputs_are_checked():
    _, _, _, adj, x = setup()
    with pytest.raises(TypeError):
        oga.tendency(adj, x[0].float(), x[1], x[2])
    with pytest.raises(TypeError):
        oga.rollout(adj, x[0].cpu(), x[1], x[2], 0.0, DT, 2)
    with pytest.raises(ValueError):
        oga.tendency(adj, x[0][:-1], x[1], x[2])


def test_state_views_share_memory():
    mesh, params, _, _, x = setup()
    S = state(mesh, params, x)
    h, vn, tr = S.as_tensors()
    vn.mul_(2.0)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(S.download()[1], 2.0 * x[1].cpu().numpy())
    np.testing.assert_array_equal(h.cpu().numpy(), x[0].cpu().numpy())
    np.testing.assert_array_equal(tr.cpu().numpy(), x[2].cpu().numpy())
