"""The oracle against golden vectors produced by the reference itself.

tests/golden/*.npz were written by tests/golden/make_golden.py, which runs
the omega_playground sources (unmodified) compiled against the host-only
Kokkos shim.  The oracle restates those sources in C in the same association
order, so everything must match bit for bit: mesh tables, every auxiliary
field and tendency of one compute_tendency, and the stepped state."""
import numpy as np
import pytest

from helpers import STEPPER_KIND, golden_names, load_golden, oracle_model

AUX = ["rvort_vertex", "norm_rvort_vertex", "norm_pvort_vertex",
       "norm_rvort_edge", "norm_pvort_edge", "mean_h_edge", "ke_cell",
       "vel_div_cell", "norm_tr_cell", "vel_del2_edge",
       "vel_del2_rvort_vertex", "vel_del2_div_cell", "tracer_del2_cell"]


@pytest.mark.parametrize("name", golden_names())
def test_mesh_tables_bit_exact(name):
    g = load_golden(name)
    m, _ = oracle_model(g["cfg"])
    for k, v in m.tables.items():
        if k in g:
            np.testing.assert_array_equal(v, g[k], err_msg=k)


@pytest.mark.parametrize("name", golden_names())
def test_tendency_and_aux_bit_exact(name):
    g = load_golden(name)
    _, md = oracle_model(g["cfg"])
    th, tv, tt = md.compute_tendency(g["in_h"].copy(), g["in_vn"].copy(),
                                     g["in_tr"].copy(), 0.0, 0)
    np.testing.assert_array_equal(th, g["tend_h"])
    np.testing.assert_array_equal(tv, g["tend_vn"])
    np.testing.assert_array_equal(tt, g["tend_tr"])
    for a in AUX:
        np.testing.assert_array_equal(md.aux(a), g[a].ravel(), err_msg=a)


@pytest.mark.parametrize("name", golden_names())
def test_steps_and_diagnostics_bit_exact(name):
    g = load_golden(name)
    cfg = g["cfg"]
    _, md = oracle_model(cfg)
    h, vn, tr = g["in_h"].copy(), g["in_vn"].copy(), g["in_tr"].copy()
    assert md.mass(h) == g["mass0"][0]
    assert md.energy(h, vn) == g["energy0"][0]
    assert md.circulation(vn) == g["circulation0"][0]
    if cfg["stepper"] in STEPPER_KIND:
        kind, ns = STEPPER_KIND[cfg["stepper"]]
        md.step(h, vn, tr, cfg["t0"], cfg["dt"], cfg["nsteps"], kind, ns)
    np.testing.assert_array_equal(h, g["h_final"])
    np.testing.assert_array_equal(vn, g["vn_final"])
    np.testing.assert_array_equal(tr, g["tr_final"])
    assert md.mass(h) == g["mass1"][0]


def test_reference_test_tables_recorded():
    """The reference's six CTest programs ran (built against the shim) and
    their pass criteria hold in the recorded output."""
    import os
    import re
    from helpers import GOLDEN
    txt = open(os.path.join(GOLDEN, "reference_tests.txt")).read()
    for t in ("operator_convergence", "nonlinear_swe_convergence",
              "double_vortex", "tracer_advection_convergence",
              "tracer_diffusion_convergence",
              "tracer_hyperdiffusion_convergence"):
        assert f"=== {t}" in txt
    m = re.search(r"Mass change: (\S+)", txt)
    assert abs(float(m.group(1))) < 5e-14
