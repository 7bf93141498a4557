"""The shallow-water tendency and a checkpointed rollout as PyTorch autograd
Functions over the C ABI's derivative entry points.

- tendency(adjoint, h, vn, tr): the model's tendency (swg_compute_tendency);
  its vjp is swg_adj_tendency (hand-written reverse mode), its jvp
  swg_tlm_tendency (dual-number forward mode).
- rollout(adjoint, h, vn, tr, t0, dt, nsteps): nsteps steps of the adjoint's
  stepper (RK4 or low-storage RK) by swg_adj_forward, which stores the
  binomial checkpoints; its vjp is swg_adj_backward, its jvp swg_tlm_apply.

h [C][K], vn [E][K] and tr [T][C][K] are float64 CUDA tensors; the results
have the same shapes.  Every call runs on torch's current stream, which
inside a backward is the stream the autograd engine picked for the node.
The reference has no derivative, so this module has no counterpart there;
it is optional glue, and the solver itself never imports torch.

One adjoint object holds the checkpoints of one rollout: a second rollout
through the same object before the first one's backward makes that backward
raise, so keep one Adjoint per live rollout graph."""
import torch

from .shallow_water import AddMode, Adjoint, ShallowWaterState

_NAMES = ("h", "vn", "tr")


def _workspace(adjoint: Adjoint, key: str, n: int):
    """n device states owned by the adjoint, made once per use."""
    ws = adjoint.__dict__.setdefault("_torch_ws", {})
    if key not in ws:
        model = adjoint.model
        ws[key] = [ShallowWaterState(model.m_mesh, model.m_params.m_ntracers)
                   for _ in range(n)]
    return ws[key]


def _check(state: ShallowWaterState, fields):
    for name, want, t in zip(_NAMES, state.shapes(), fields):
        if not isinstance(t, torch.Tensor) or not t.is_cuda or \
                t.dtype != torch.float64:
            raise TypeError(f"{name}: expected a float64 CUDA tensor")
        if tuple(t.shape) != tuple(want):
            raise ValueError(f"{name}: shape {tuple(t.shape)}, expected "
                             f"{tuple(want)}")


def _load(state: ShallowWaterState, fields):
    for dst, src in zip(state.as_tensors(), fields):
        if src is None:
            dst.zero_()
        else:
            dst.copy_(src)


def _take(state: ShallowWaterState):
    return tuple(t.clone() for t in state.as_tensors())


def _stream():
    return torch.cuda.current_stream().cuda_stream


class Tendency(torch.autograd.Function):
    """dx/dt = f(x) at time t (the adjoint's model; no forcing hook)."""

    @staticmethod
    def forward(ctx, adjoint, t, h, vn, tr):
        x, tend = _workspace(adjoint, "tendency", 2)
        _check(x, (h, vn, tr))
        _load(x, (h, vn, tr))
        adjoint.model.compute_tendency(tend, x, t, AddMode.replace,
                                       stream=_stream())
        ctx.adjoint = adjoint
        ctx.save_for_backward(h, vn, tr)
        ctx.save_for_forward(h, vn, tr)
        return _take(tend)

    @staticmethod
    @torch.autograd.function.once_differentiable
    def backward(ctx, gh, gvn, gtr):
        adjoint = ctx.adjoint
        x, mu, lam = _workspace(adjoint, "tendency_vjp", 3)
        _load(x, ctx.saved_tensors)
        _load(mu, (gh, gvn, gtr))
        adjoint.adj_tendency(x, mu, lam, stream=_stream())
        return (None, None) + _take(lam)

    @staticmethod
    def jvp(ctx, _adjoint, _t, dh, dvn, dtr):
        adjoint = ctx.adjoint
        x, dx, dtend = _workspace(adjoint, "tendency_jvp", 3)
        _load(x, ctx.saved_tensors)
        _load(dx, (dh, dvn, dtr))
        adjoint.tlm_tendency(x, dx, dtend, stream=_stream())
        return _take(dtend)


class Rollout(torch.autograd.Function):
    """x_N after nsteps steps of size dt from x_0 = (h, vn, tr) at t0."""

    @staticmethod
    def forward(ctx, adjoint, t0, dt, nsteps, h, vn, tr):
        x0, xn = _workspace(adjoint, "rollout", 2)
        _check(x0, (h, vn, tr))
        _load(x0, (h, vn, tr))
        adjoint.forward(x0, t0, dt, nsteps, xn, stream=_stream())
        gen = adjoint.__dict__.get("_torch_gen", 0) + 1
        adjoint._torch_gen = gen
        ctx.adjoint, ctx.gen, ctx.args = adjoint, gen, (t0, dt, nsteps)
        ctx.save_for_forward(h, vn, tr)
        return _take(xn)

    @staticmethod
    @torch.autograd.function.once_differentiable
    def backward(ctx, gh, gvn, gtr):
        adjoint = ctx.adjoint
        if adjoint.__dict__.get("_torch_gen") != ctx.gen:
            raise RuntimeError(
                "rollout backward: the adjoint's checkpoints belong to a "
                "later rollout or were used by an earlier backward; keep one "
                "Adjoint per live rollout graph")
        adjoint._torch_gen = ctx.gen + 1          # the sweep consumes them
        (lam,) = _workspace(adjoint, "rollout_vjp", 1)
        _load(lam, (gh, gvn, gtr))
        adjoint.backward(lam, stream=_stream())
        return (None, None, None, None) + _take(lam)

    @staticmethod
    def jvp(ctx, _adjoint, _t0, _dt, _nsteps, dh, dvn, dtr):
        adjoint = ctx.adjoint
        x0, dx = _workspace(adjoint, "rollout_jvp", 2)
        _load(x0, ctx.saved_tensors)
        _load(dx, (dh, dvn, dtr))
        t0, dt, nsteps = ctx.args
        adjoint.tlm_apply(x0, dx, t0, dt, nsteps, stream=_stream())
        return _take(dx)


def tendency(adjoint: Adjoint, h, vn, tr, t: float = 0.0):
    """The tendency (h_tend, vn_tend, tr_tend) of the adjoint's model."""
    return Tendency.apply(adjoint, float(t), h, vn, tr)


def rollout(adjoint: Adjoint, h, vn, tr, t0: float, dt: float, nsteps: int):
    """The state after nsteps steps of the adjoint's stepper."""
    return Rollout.apply(adjoint, float(t0), float(dt), int(nsteps), h, vn,
                         tr)
