"""Configurations crossed with the stepping paths.

A model's enabled set (h or vn frozen, no or 12 tracers, each dissipation
term alone) changes which passes run and which buffers a stage reads, so every
path is run on each:
- the steppers (RK4, LSRK5, Euler) against the oracle, 3 steps, <= 1e-12;
- batches of such members, bitwise equal to each member stepped alone;
- the adjoint's tendency and 6-step trajectory dot products against the
  tangent-linear model, <= 1e-12, and its forward sweep's x_N bitwise equal
  to the plain stepper's;
- the host-state stepper, bitwise equal to upload + step + download.
(The allocation-free tendency takes the same sets in test_zz_no_alloc.py.)"""
import numpy as np
import pytest

import omega_playground_gb300 as og
import pyoracle
from helpers import rel_diff
from omega_playground_gb300.workloads import uniform

pytestmark = pytest.mark.gpu

TOL = 1e-12
ALL = dict(f0=1e-4, grav=9.81, visc_del2=1e3, visc_del4=1e9, eddy_diff2=1e3,
           eddy_diff4=1e9)
CONFIGS = {
    "h_frozen": dict(ALL, disable_h=True),
    "vn_frozen": dict(ALL, disable_vn=True),
    "no_tracers": dict(ALL, T=0),
    "del2_only": dict(f0=1e-4, grav=9.81, visc_del2=1e3, eddy_diff2=1e3),
    "del4_only": dict(f0=1e-4, grav=9.81, visc_del4=1e9, eddy_diff4=1e9),
    "tracer_del4_only": dict(f0=1e-4, grav=9.81, eddy_diff4=1e9),
    "inviscid": dict(f0=1e-4, grav=9.81),
    "many_tracers": dict(ALL, T=12),
}
STEPPERS = [("rk4", 4), ("lsrk", 5), ("lsrk", 1)]


def build(nx, ny, K, cfg):
    c = dict(cfg)
    T = c.pop("T", 2)
    dh, dv = c.pop("disable_h", False), c.pop("disable_vn", False)
    mesh = og.PlanarHexagonalMesh(nx, ny, 1e4, K)
    params = og.ShallowWaterParams(
        m_f0=c.get("f0", 0.0), m_grav=c.get("grav", 9.81),
        m_visc_del2=c.get("visc_del2", 0.0), m_visc_del4=c.get("visc_del4", 0.0),
        m_eddy_diff2=c.get("eddy_diff2", 0.0),
        m_eddy_diff4=c.get("eddy_diff4", 0.0), m_ntracers=T,
        m_disable_h_tendency=dh, m_disable_vn_tendency=dv)
    om = pyoracle.OracleMesh(nx, ny, 1e4, K)
    omd = pyoracle.OracleModel(om, ntracers=T, disable_h_tendency=dh,
                               disable_vn_tendency=dv, **c)
    return mesh, params, og.ShallowWaterModel(mesh, params), omd


def state(mesh, T, seed):
    C_, E, K = mesh.m_ncells, mesh.m_nedges, mesh.m_nlayers
    h = 1000.0 + 3.0 * uniform(seed, C_ * K).reshape(C_, K)
    vn = 0.2 * (uniform(seed + 1, E * K).reshape(E, K) - 0.5)
    tr = h[None] * (0.5 + uniform(seed + 2, T * C_ * K).reshape(T, C_, K))
    return h, vn, tr


@pytest.mark.parametrize("kind,nstages", STEPPERS)
@pytest.mark.parametrize("name", ["h_frozen", "vn_frozen", "no_tracers",
                                  "tracer_del4_only", "many_tracers"])
def test_steppers_against_oracle(name, kind, nstages):
    mesh, params, model, omd = build(10, 8, 4, CONFIGS[name])
    T = params.m_ntracers
    x = state(mesh, T, 17)
    want = omd.step(*(a.copy() for a in x), 0.0, 20.0, 3, kind=kind,
                    nstages=nstages)
    for use_graph in (False, True):
        S = og.ShallowWaterState(mesh, params)
        S.upload(*x)
        st = og.RK4Stepper(model) if kind == "rk4" else og.LSRKStepper(model,
                                                                       nstages)
        st.step(S, 0.0, 20.0, 3, use_graph=use_graph)
        for g, w in zip(S.download(), want):
            if w.size:
                assert rel_diff(g, w) <= TOL, (name, kind, nstages)
    if name == "h_frozen":
        np.testing.assert_array_equal(S.download()[0], x[0])
    if name == "vn_frozen":
        np.testing.assert_array_equal(S.download()[1], x[1])


@pytest.mark.parametrize("kind,nstages", STEPPERS)
def test_batch_of_mixed_configurations(kind, nstages):
    members = []
    for j, name in enumerate(CONFIGS):
        mesh, params, model, _ = build(6 + 2 * (j % 3), 6 + 2 * (j % 2),
                                       3 + j, CONFIGS[name])
        members.append((mesh, params, model,
                        state(mesh, params.m_ntracers, 50 + 3 * j)))
    singles = []
    for mesh, params, model, x in members:
        S = og.ShallowWaterState(mesh, params)
        S.upload(*x)
        st = og.RK4Stepper(model) if kind == "rk4" else og.LSRKStepper(model,
                                                                       nstages)
        st.step(S, 0.0, 20.0, 3, use_graph=False)
        singles.append(S.download())
    for cfg in range(og.Batch.config_count()):
        states = []
        for mesh, params, model, x in members:
            S = og.ShallowWaterState(mesh, params)
            S.upload(*x)
            states.append(S)
        b = og.Batch([m[2] for m in members], states, kind, nstages)
        b.set_config(cfg)
        b.step(0.0, 20.0, 3)
        for m, (S, want) in enumerate(zip(states, singles)):
            for g, w in zip(S.download(), want):
                np.testing.assert_array_equal(g, w, err_msg=f"{cfg} {m}")


def dot(a, b):
    return sum(float(np.sum(p * q)) for p, q in zip(a, b))


@pytest.mark.parametrize("kind,nstages", [("rk4", 4), ("lsrk", 5)])
@pytest.mark.parametrize("name", list(CONFIGS))
def test_adjoint_dot_products(name, kind, nstages):
    mesh, params, model, _ = build(10, 8, 3, CONFIGS[name])
    T = params.m_ntracers
    adj = og.Adjoint(model, 2, kind, nstages)
    x = state(mesh, T, 71)
    dx = tuple(s * (uniform(80 + j, a.size).reshape(a.shape) - 0.5)
               for j, (a, s) in enumerate(zip(x, (1.0, 0.01, 10.0))))
    mu = tuple(uniform(90 + j, a.size).reshape(a.shape) - 0.5
               for j, a in enumerate(x))

    def mk(a):
        st = og.ShallowWaterState(mesh, params)
        st.upload(*a)
        return st

    X = mk(x)
    JD, JT = og.ShallowWaterState(mesh, params), og.ShallowWaterState(mesh, params)
    adj.tlm_tendency(X, mk(dx), JD)
    adj.adj_tendency(X, mk(mu), JT)
    lhs, rhs = dot(JD.download(), mu), dot(dx, JT.download())
    assert abs(lhs - rhs) <= TOL * max(abs(lhs), abs(rhs), 1e-300), (lhs, rhs)
    XN = og.ShallowWaterState(mesh, params)
    adj.forward(X, 0.0, 20.0, 6, XN)
    LAM = mk(mu)
    adj.backward(LAM)
    DX = mk(dx)
    adj.tlm_apply(X, DX, 0.0, 20.0, 6)
    lhs, rhs = dot(DX.download(), mu), dot(dx, LAM.download())
    assert abs(lhs - rhs) <= TOL * max(abs(lhs), abs(rhs)), (lhs, rhs)
    ref = mk(x)
    st = og.RK4Stepper(model) if kind == "rk4" else og.LSRKStepper(model,
                                                                   nstages)
    st.step(ref, 0.0, 20.0, 6, use_graph=False)
    for g, w in zip(XN.download(), ref.download()):
        np.testing.assert_array_equal(g, w)


@pytest.mark.parametrize("name", list(CONFIGS))
def test_host_stepper(name):
    """The host-state stepper (chunks of 2 of 5 levels) on each enabled
    set, bitwise equal to upload + step + download."""
    mesh, params, model, _ = build(10, 8, 5, CONFIGS[name])
    T = params.m_ntracers
    x = state(mesh, T, 33)
    for kind, nstages in STEPPERS:
        S = og.ShallowWaterState(mesh, params)
        S.upload(*x)
        st = og.RK4Stepper(model) if kind == "rk4" else og.LSRKStepper(model,
                                                                       nstages)
        st.step(S, 0.0, 20.0, 3)
        hs = og.HostStepper(model, kind, nstages, 2)
        arrs = hs.pinned_state()
        for a, b in zip(arrs, x):
            if a.size:
                a[...] = b
        hs.step(*arrs, 0.0, 20.0, 3)
        for g, w in zip(arrs, S.download()):
            np.testing.assert_array_equal(g, w, err_msg=f"{name} {kind}")


@pytest.mark.parametrize("kind,nstages", [("rk4", 4), ("lsrk", 5)])
def test_batch_of_general_meshes(kind, nstages):
    """Members on perturbed general MPAS tables (10 nonzero TRiSK weights,
    so the 10-wide edges-on-edge kernels; random 0/1 edge masks, scaling and
    5-edge cells), bitwise equal to each member stepped alone, in every
    launch configuration."""
    from test_general_mesh_gpu import general_mesh, models
    from test_general_mesh_gpu import state as gstate
    members = []
    for j, (nx, ny, K, T) in enumerate(((10, 8, 5, 2), (6, 6, 9, 1),
                                        (8, 10, 3, 3))):
        om, gm = general_mesh(nx, ny, K, 300 + j)
        _, gp, model = models(om, gm, T)
        members.append((gm, gp, model, gstate(om, T, 400 + j)))
    singles = []
    for gm, gp, model, x in members:
        S = og.ShallowWaterState(gm, gp)
        S.upload(*x)
        st = og.RK4Stepper(model) if kind == "rk4" else og.LSRKStepper(model,
                                                                       nstages)
        st.step(S, 0.0, 5.0, 3, use_graph=False)
        singles.append(S.download())
    for cfg in range(og.Batch.config_count()):
        states = []
        for gm, gp, model, x in members:
            S = og.ShallowWaterState(gm, gp)
            S.upload(*x)
            states.append(S)
        b = og.Batch([m[2] for m in members], states, kind, nstages)
        b.set_config(cfg)
        b.step(0.0, 5.0, 3)
        for m, (S, want) in enumerate(zip(states, singles)):
            for g, w in zip(S.download(), want):
                assert np.all(np.isfinite(w))
                np.testing.assert_array_equal(g, w, err_msg=f"{cfg} {m}")


@pytest.mark.parametrize("kind,nstages", [("rk4", 4), ("lsrk", 5)])
def test_forcing_hook_on_a_frozen_field(kind, nstages):
    """The forcing hook with h frozen adds c to h's tendency.  The reference
    zeroes a tendency only inside that field's compute_*_tendency
    (shallow_water_model.cpp:52-60, 323-345), so a frozen field's tendency is
    never reset and the hook's additions accumulate over evaluations:
    - RK4 (rk4.cpp:28-104, four evaluations per step, replace mode): the
      e-th evaluation leaves e*c, so a step adds dt*c*sum_s b_s*(4n+s+1);
    - LSRK (tendency scaled by a_s, then incremented): exactly dt*c a step.
    The GPU reproduces both (absolute error <= 1e-10 on h ~ 1000)."""
    torch = pytest.importorskip("torch")
    from omega_playground_gb300.shallow_water import _DeviceArray
    mesh, params, _, _ = build(8, 6, 3, CONFIGS["h_frozen"])
    C_, K = mesh.m_ncells, mesh.m_nlayers
    c, dt, n = 1e-3, 20.0, 4

    class Forced(og.ShallowWaterModel):
        def additional_tendency(self, h_tend, vn_tend, h, vn, t, stream):
            torch.as_tensor(_DeviceArray(None, h_tend, (C_, K)),
                            device="cuda").add_(c)

    model = Forced(mesh, params)
    x = state(mesh, params.m_ntracers, 61)
    S = og.ShallowWaterState(mesh, params)
    S.upload(*x)
    st = og.RK4Stepper(model) if kind == "rk4" else og.LSRKStepper(model,
                                                                   nstages)
    st.step(S, 0.0, dt, n)
    torch.cuda.synchronize()
    if kind == "rk4":
        b = (1 / 6, 1 / 3, 1 / 3, 1 / 6)
        rise = dt * c * sum(b[s] * (4 * j + s + 1) for j in range(n)
                            for s in range(4))
    else:
        rise = n * dt * c
    got = S.download()[0] - x[0]
    # h ~ 1000: round-off of the updates is ~1e-13 absolute
    assert np.max(np.abs(got - rise)) <= 1e-10, (got.min(), got.max(), rise)


def test_paths_on_a_caller_stream():
    """Every stepping path launched on a non-blocking stream of the
    caller's (fork/join branches, graph replays, the adjoint's advance
    stream and the batch's launches must order against it): results
    bitwise equal to the same calls on the legacy stream."""
    torch = pytest.importorskip("torch")
    s = torch.cuda.Stream()
    sp = s.cuda_stream
    mesh, params, model, _ = build(10, 8, 5, CONFIGS["many_tracers"])
    T = params.m_ntracers
    x = state(mesh, T, 5)

    def run(stream):
        out = {}
        S = og.ShallowWaterState(mesh, params)
        S.upload(*x, stream=stream)
        og.LSRKStepper(model, 5).step(S, 0.0, 20.0, 3, stream=stream)
        og.RK4Stepper(model).step(S, 0.0, 20.0, 2, stream=stream)
        out["steps"] = S.download(stream=stream)
        Tn = og.ShallowWaterState(mesh, params)
        model.compute_tendency(Tn, S, 0.0, stream=stream)
        out["tend"] = Tn.download(stream=stream)
        adj = og.Adjoint(model, 2)
        XN = og.ShallowWaterState(mesh, params)
        adj.forward(S, 0.0, 20.0, 5, XN, stream=stream)
        L = og.ShallowWaterState(mesh, params)
        L.upload(*state(mesh, T, 9), stream=stream)
        adj.backward(L, stream=stream)
        out["grad"] = L.download(stream=stream)
        B = og.ShallowWaterState(mesh, params)
        B.upload(*x, stream=stream)
        b = og.Batch([model], [B], "lsrk", 5)
        b.step(0.0, 20.0, 3, stream=stream)
        out["batch"] = B.download(stream=stream)
        return out

    ref = run(None)
    got = run(sp)
    for k in ref:
        for a, bb in zip(got[k], ref[k]):
            np.testing.assert_array_equal(a, bb, err_msg=k)


def test_batch_of_many_small_members():
    """300 members of 1 to 4x4 cells, 1 to 6 levels, 0 to 3 tracers: the
    member table and the per-pass block prefixes at that count, bitwise
    against each member stepped alone, persistent and per-pass shapes."""
    members = []
    for j in range(300):
        nx, ny = 1 + j % 4, 1 + (j // 4) % 4
        cfg = dict(CONFIGS["many_tracers"], T=j % 4)
        mesh, params, model, _ = build(nx, ny, 1 + j % 6, cfg)
        members.append((mesh, params, model,
                        state(mesh, params.m_ntracers, 1000 + 3 * j)))
    singles = []
    for mesh, params, model, x in members:
        S = og.ShallowWaterState(mesh, params)
        S.upload(*x)
        og.LSRKStepper(model, 5).step(S, 0.0, 20.0, 2, use_graph=False)
        singles.append(S.download())
    for cfg in (0, og.Batch.config_count() - 1):
        states = []
        for mesh, params, model, x in members:
            S = og.ShallowWaterState(mesh, params)
            S.upload(*x)
            states.append(S)
        b = og.Batch([m[2] for m in members], states, "lsrk", 5)
        b.set_config(cfg)
        b.step(0.0, 20.0, 2)
        for m, (S, want) in enumerate(zip(states, singles)):
            for g, w in zip(S.download(), want):
                np.testing.assert_array_equal(g, w, err_msg=f"{cfg} {m}")


@pytest.mark.parametrize("kind,nstages", STEPPERS)
def test_checkpoint_and_resume_is_bitwise(kind, nstages, tmp_path):
    """Stopping after 3 steps, saving the state to disk (download + npz),
    and resuming 3 more steps in a new process-like setup (fresh mesh,
    model, state and stepper) equals 6 uninterrupted steps bit for bit: the
    steppers carry nothing across steps but the state (LSRK's first stage
    has a = 0)."""
    mesh, params, model, _ = build(10, 8, 4, CONFIGS["many_tracers"])
    T = params.m_ntracers
    x = state(mesh, T, 3)

    def stepper(m):
        return og.RK4Stepper(m) if kind == "rk4" else og.LSRKStepper(m, nstages)

    S = og.ShallowWaterState(mesh, params)
    S.upload(*x)
    stepper(model).step(S, 0.0, 20.0, 6)
    want = S.download()
    S.upload(*x)
    stepper(model).step(S, 0.0, 20.0, 3)
    h, vn, tr = S.download()
    np.savez(tmp_path / "ckpt.npz", h=h, vn=vn, tr=tr)
    del S
    mesh2, params2, model2, _ = build(10, 8, 4, CONFIGS["many_tracers"])
    ck = np.load(tmp_path / "ckpt.npz")
    R = og.ShallowWaterState(mesh2, params2)
    R.upload(ck["h"], ck["vn"], ck["tr"])
    stepper(model2).step(R, 60.0, 20.0, 3)
    for g, w in zip(R.download(), want):
        np.testing.assert_array_equal(g, w)


def test_every_small_mesh():
    """Every mesh of nx, ny in 1..12 cells (odd rows, one-cell-wide meshes,
    every term on, 2 levels, 2 tracers): the GPU tendency against the
    oracle, <= 1e-12, and the adjoint tendency's dot product against the
    tangent-linear model, <= 1e-12 of the sum of the products' magnitudes.
    On one-cell-wide meshes an edge has the same cell on both sides and its
    difference terms cancel, exactly in the tangent-linear model and to
    round-off in the adjoint, so the dot product itself can be far below
    its terms and is not the scale."""
    for nx in range(1, 13):
        for ny in range(1, 13):
            mesh, params, model, omd = build(nx, ny, 2, ALL)
            x = state(mesh, 2, 10 * nx + ny)
            want = omd.compute_tendency(*x)
            S = og.ShallowWaterState(mesh, params)
            S.upload(*x)
            Tn = og.ShallowWaterState(mesh, params)
            model.compute_tendency(Tn, S, 0.0)
            for g, w in zip(Tn.download(), want):
                assert rel_diff(g, w) <= TOL, (nx, ny)
            adj = og.Adjoint(model, 1)
            dx = tuple(s * (uniform(7 * nx + ny, a.size).reshape(a.shape)
                            - 0.5) for a, s in zip(x, (1.0, 0.01, 10.0)))
            mu = tuple(uniform(9 * nx + ny + j, a.size).reshape(a.shape)
                       - 0.5 for j, a in enumerate(x))
            DX, MU = og.ShallowWaterState(mesh, params), \
                og.ShallowWaterState(mesh, params)
            DX.upload(*dx)
            MU.upload(*mu)
            JD, JT = og.ShallowWaterState(mesh, params), \
                og.ShallowWaterState(mesh, params)
            adj.tlm_tendency(S, DX, JD)
            adj.adj_tendency(S, MU, JT)
            jd, jt = JD.download(), JT.download()
            lhs, rhs = dot(jd, mu), dot(dx, jt)
            scale = max(sum(float(np.sum(np.abs(p * q)))
                            for p, q in zip(jd, mu)),
                        sum(float(np.sum(np.abs(p * q)))
                            for p, q in zip(dx, jt)))
            assert abs(lhs - rhs) <= TOL * scale, (nx, ny, lhs, rhs, scale)
