"""The model's auxiliary state and per-field tendencies (the reference's
m_aux_state.compute and compute_h_tendency / compute_vn_tendency /
compute_tr_tendency, shallow_water_auxstate.cpp:12-50 and
shallow_water_model.cpp:43-311), through the C ABI against the oracle's
restatement of the same routines, <= 1e-12.

The per-field calls read the last auxiliary state and their own arguments,
so the tests compute the auxiliary state of one state (A) and pass another
(B) as the arguments: the thickness flux then mixes A's mean thickness with
B's normal velocity, exactly as the reference's functors do."""
import ctypes as C

import numpy as np
import pytest

import omega_playground_gb300 as og
from helpers import load_golden, oracle_model, rel_diff
from omega_playground_gb300 import _capi

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _setup(cfg, cls=og.ShallowWaterModel):
    mesh = og.PlanarHexagonalMesh(cfg["nx"], cfg["ny"], cfg["dc"], cfg["K"])
    params = og.ShallowWaterParams(
        m_f0=cfg["f0"], m_grav=cfg["grav"], m_visc_del2=cfg["visc_del2"],
        m_visc_del4=cfg["visc_del4"], m_eddy_diff2=cfg["eddy_diff2"],
        m_eddy_diff4=cfg["eddy_diff4"], m_ntracers=cfg["T"],
        m_disable_h_tendency=cfg.get("disable_h", False),
        m_disable_vn_tendency=cfg.get("disable_vn", False))
    return mesh, params, cls(mesh, params)


def _states(g, seed):
    """State A (the golden input) and a perturbed state B."""
    rng = np.random.default_rng(seed)
    a = [g["in_h"].copy(), g["in_vn"].copy(), g["in_tr"].copy()]
    b = [a[0] * (1 + 1e-3 * rng.standard_normal(a[0].shape)),
         a[1] + 0.05 * rng.standard_normal(a[1].shape),
         a[2] * (1 + 0.1 * rng.standard_normal(a[2].shape))]
    return a, b


def _device(mesh, params, arrays):
    s = og.ShallowWaterState(mesh, params)
    s.upload(*arrays)
    return s


@pytest.mark.parametrize("add_mode", [0, 1])
@pytest.mark.parametrize("golden", ["rk4_all_terms", "lsrk5_all_terms"])
def test_field_tendencies_match_oracle(golden, add_mode):
    g = load_golden(golden)
    cfg = g["cfg"]
    A, B = _states(g, 7)
    mesh, params, model = _setup(cfg)
    SA, SB = _device(mesh, params, A), _device(mesh, params, B)
    ah, avn, atr = SA.device_ptrs()
    bh, bvn, btr = SB.device_ptrs()
    # the tendencies start from a nonzero field (increment adds to it)
    rng = np.random.default_rng(3)
    T0 = [rng.standard_normal(x.shape) for x in A]
    TEND = _device(mesh, params, T0)
    th, tv, tt = TEND.device_ptrs()
    model.compute_aux(ah, avn, atr)
    model.compute_h_tendency(th, bh, bvn, add_mode)
    model.compute_vn_tendency(tv, bh, bvn, add_mode)
    model.compute_tr_tendency(tt, btr, bvn, add_mode)
    got = TEND.download()

    om, md = oracle_model(cfg)
    md.compute_aux(*A)
    ref = [x.copy() for x in T0]
    md.compute_h_tendency(ref[0], B[1], add_mode)
    md.compute_vn_tendency(ref[1], B[0], B[1], add_mode)
    md.compute_tr_tendency(ref[2], B[1], add_mode)
    for name, a, b in zip(("h", "vn", "tr"), got, ref):
        assert rel_diff(a, b) <= TOL, (name, rel_diff(a, b))
    # the mixed flux matters: B's arguments give a different result from a
    # tendency evaluated at B
    full = md.compute_tendency(*B, add_mode=0)
    assert rel_diff(ref[1] - (T0[1] if add_mode else 0), full[1]) > 1e-6


def test_per_field_after_compute_tendency_equals_it_bitwise():
    """After compute_tendency(state), the per-field calls with the same
    state's fields reproduce its three outputs bit for bit (the auxiliary
    state is the evaluation's)."""
    g = load_golden("rk4_all_terms")
    mesh, params, model = _setup(g["cfg"])
    S = _device(mesh, params, [g["in_h"], g["in_vn"], g["in_tr"]])
    full = og.ShallowWaterState(mesh, params)
    model.compute_tendency(full, S, 0.0)
    ref = full.download()
    h, vn, tr = S.device_ptrs()
    T = og.ShallowWaterState(mesh, params)
    th, tv, tt = T.device_ptrs()
    model.compute_h_tendency(th, h, vn)
    model.compute_vn_tendency(tv, h, vn)
    model.compute_tr_tendency(tt, tr, vn)
    for a, b in zip(T.download(), ref):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("term", [0, 1, 3, 4, 6, 8])
def test_field_tendencies_follow_term_switches(term):
    g = load_golden("lsrk5_all_terms")
    cfg = g["cfg"]
    A, B = _states(g, 11)
    mesh, params, model = _setup(cfg)
    from omega_playground_gb300.shallow_water import TERMS
    getattr(model, TERMS[term]).m_enabled = False
    SA, SB = _device(mesh, params, A), _device(mesh, params, B)
    TEND = og.ShallowWaterState(mesh, params)
    th, tv, tt = TEND.device_ptrs()
    model.m_aux_state.compute(*SA.device_ptrs())
    bh, bvn, btr = SB.device_ptrs()
    model.compute_h_tendency(th, bh, bvn)
    model.compute_vn_tendency(tv, bh, bvn)
    model.compute_tr_tendency(tt, btr, bvn)
    om, md = oracle_model(cfg)
    md.set_term(term, False)
    md.compute_aux(*A)
    ref = [np.zeros_like(x) for x in A]
    md.compute_h_tendency(ref[0], B[1])
    md.compute_vn_tendency(ref[1], B[0], B[1])
    md.compute_tr_tendency(ref[2], B[1])
    for a, b in zip(TEND.download(), ref):
        assert rel_diff(a, b) <= TOL


def test_aux_state_view_matches_oracle():
    """m_aux_state's reference-named members after an auxiliary
    computation: mean / flux thickness, relative vorticity, kinetic energy,
    divergence and normalised tracers equal the oracle's; the summed
    vorticity members equal the sums of the oracle's split members."""
    g = load_golden("rk4_all_terms")
    cfg = g["cfg"]
    A, _ = _states(g, 5)
    mesh, params, model = _setup(cfg)
    SA = _device(mesh, params, A)
    model.compute_aux(*SA.device_ptrs())
    aux = model.m_aux_state
    om, md = oracle_model(cfg)
    md.compute_aux(*A)
    th, vo, ki, tr = (aux.m_thickness_aux, aux.m_vorticity_aux,
                      aux.m_kinetic_aux, aux.m_tracer_aux)
    pairs = [(th.m_mean_h_edge, md.aux("mean_h_edge")),
             (th.m_flux_h_edge, md.aux("flux_h_edge")),
             (vo.m_rvort_vertex, md.aux("rvort_vertex")),
             (vo.m_pv_vertex, md.aux("norm_rvort_vertex")
              + md.aux("norm_pvort_vertex")),
             (vo.m_pv_edge, 2 * (md.aux("norm_rvort_edge")
                                 + md.aux("norm_pvort_edge"))),
             (ki.m_ke_cell, md.aux("ke_cell")),
             (ki.m_vel_div_cell, md.aux("vel_div_cell")),
             (tr.m_norm_tr_cell, md.aux("norm_tr_cell"))]
    for got, ref in pairs:
        assert got is not None
        assert rel_diff(got.ravel(), ref) <= TOL
    assert tr.m_norm_tr_cell.shape == (cfg["T"], mesh.m_ncells, cfg["K"])


def test_linear_model_fields_and_refusals():
    """The linear model's per-field calls read h and vn directly (no
    auxiliary state) and equal the oracle's linear tendency; a model with the
    velocity tendency disabled refuses the velocity call (it keeps no
    velocity intermediates); bad add modes are refused."""
    g = load_golden("rk4_all_terms")
    cfg = dict(g["cfg"], T=0, visc_del2=0.0, visc_del4=0.0, eddy_diff2=0.0,
               eddy_diff4=0.0)
    mesh = og.PlanarHexagonalMesh(cfg["nx"], cfg["ny"], cfg["dc"], cfg["K"])
    lp = og.LinearShallowWaterParams(m_f0=cfg["f0"], m_grav=cfg["grav"],
                                     m_h0=1000.0)
    lin = og.LinearShallowWaterModel(mesh, lp)
    h, vn = g["in_h"] - 1000.0, g["in_vn"]
    S = _device(mesh, lp, [h, vn, None])
    T = og.ShallowWaterState(mesh, lp)
    sh, sv, _ = S.device_ptrs()
    th, tv, _ = T.device_ptrs()
    lin.compute_h_tendency(th, sh, sv)
    lin.compute_vn_tendency(tv, sh, sv)
    with pytest.raises(og.SwgError):
        lin.compute_aux(sh, sv)
    import pyoracle
    om = pyoracle.OracleMesh(cfg["nx"], cfg["ny"], cfg["dc"], cfg["K"])
    md = pyoracle.OracleModel(om, f0=cfg["f0"], grav=cfg["grav"],
                              linear_h0=1000.0)
    ref = md.compute_tendency(h.copy(), vn.copy(), None)
    got = T.download()
    assert rel_diff(got[0], ref[0]) <= TOL
    assert rel_diff(got[1], ref[1]) <= TOL

    cfg2 = dict(g["cfg"], disable_vn=True)
    mesh2, params2, frozen = _setup(cfg2)
    S2 = _device(mesh2, params2, [g["in_h"], g["in_vn"], g["in_tr"]])
    T2 = og.ShallowWaterState(mesh2, params2)
    h2, v2, t2 = S2.device_ptrs()
    o2 = T2.device_ptrs()
    frozen.compute_aux(h2, v2, t2)
    with pytest.raises(og.SwgError) as e:
        frozen.compute_vn_tendency(o2[1], h2, v2)
    assert e.value.code == 6
    with pytest.raises(og.SwgError) as e:
        frozen.compute_h_tendency(o2[0], h2, v2, add_mode=2)
    assert e.value.code == 1
    lib = _capi.lib()
    assert lib.swg_compute_vn_tendency(frozen.handle, C.c_void_p(o2[1]), None,
                                       C.c_void_p(v2), 0, None) == 1
