"""The reference's six CTest programs and its benchmark driver, re-hosted on
the C++ drop-in classes (tests/cpp/*.cu over libswgpu.so), run on the GPU.

Each program applies the reference test's own pass criterion (convergence
rate within 0.05, conservation bounds) and exits non-zero otherwise.  In
addition its error table must reproduce the one the reference printed
(tests/golden/reference_tests.txt, 6 significant digits)."""
import os
import re
import subprocess

import pytest

from helpers import GOLDEN
from omega_playground_gb300 import _build

pytestmark = pytest.mark.gpu

BIN = os.path.join(_build.LIBDIR, "bin")


def reference_tables():
    txt = open(os.path.join(GOLDEN, "reference_tests.txt")).read()
    out = {}
    for block in txt.split("=== ")[1:]:
        name, body = block.split("\n", 1)
        out[name.strip()] = body
    return out


def errors(text, header):
    """Error column of the table that follows `header`."""
    lines = text.split(header, 1)[1].strip().splitlines()
    vals = []
    for ln in lines:
        parts = ln.split()
        if len(parts) < 2 or not parts[0].isdigit():
            break
        vals.append(float(parts[1]))
    return vals


def run(*args, timeout=600):
    if not os.path.exists(os.path.join(BIN, args[0])):
        _build.build_cpp_programs()
    r = subprocess.run([os.path.join(BIN, args[0]), *args[1:]],
                       capture_output=True, text=True, timeout=timeout)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


@pytest.mark.parametrize("prog,args,ref,header", [
    ("nonlinear_swe_convergence", [], "nonlinear_swe_convergence",
     "Manufactured solution convergence"),
    ("tracer_convergence", ["advection"], "tracer_advection_convergence",
     "Tracer advection convergence"),
    ("tracer_convergence", ["diffusion"], "tracer_diffusion_convergence",
     "Tracer diffusion convergence"),
    ("tracer_convergence", ["hyperdiffusion"],
     "tracer_hyperdiffusion_convergence", "Tracer hyperdiffusion convergence"),
])
def test_convergence_matches_reference(prog, args, ref, header):
    out = run(prog, *args)
    got = errors(out, header)
    want = errors(reference_tables()[ref], header)
    assert len(got) == len(want) == 2
    for g, w in zip(got, want):
        assert abs(g - w) <= 5e-6 * abs(w), (got, want)


def test_operator_convergence_matches_reference():
    out = run("operator_convergence")
    ref = reference_tables()["operator_convergence"]
    for header in ("Gradient convergence", "Divergence convergence",
                   "Curl convergence", "Reconstruction convergence"):
        got, want = errors(out, header), errors(ref, header)
        assert len(got) == len(want) == 5
        for g, w in zip(got, want):
            assert abs(g - w) <= 5e-6 * abs(w), (header, got, want)


def test_double_vortex_conservation():
    """Odd ny = 29 mesh (the reference's racy construction, reproduced in
    its serial order); bounds from test/double_vortex.cpp:159-167."""
    out = run("double_vortex")
    vals = {k: float(v) for k, v in re.findall(r"(\w+) change: (\S+)", out)}
    assert abs(vals["Mass"]) < 5e-14
    assert abs(vals["Circulation"]) < 5e-14
    assert abs(vals["Energy"]) < 1e-10


def test_benchmark_driver_runs():
    out = run("benchmark", "64", "16", "1", "4")
    m = re.search(r"updates_per_s=(\S+)", out)
    assert m and float(m.group(1)) > 0


def test_cpp_gradient_and_ensemble_classes():
    """The C++ drop-in's CheckpointedAdjoint (dot product against the
    tangent-linear model, 10 RK4 steps, every term on, <= 1e-12) and
    EnsembleStepper and HostStepper (three uneven members bitwise equal to
    RK4Stepper), and CheckpointedAdjointEnsemble (three members in two
    lockstep groups bitwise equal to their own adjoints)."""
    out = run("gradients_and_ensembles")
    assert "PASS" in out, out
    rel = float(re.search(r"rel=(\S+)", out).group(1))
    assert rel <= 1e-12
    assert "ensemble max_abs_diff=0.000e+00" in out
    assert "host max_abs_diff=0.000e+00" in out
    assert "adjoint ensemble groups=2 bitwise=1" in out


def test_cpp_term_members_and_f_vertex():
    """The C++ drop-in's nine tendency-term members: each switched off
    alone changes only the fields its term writes, reads back false, equals
    the same term switched through the C ABI bit for bit, and switching it
    back restores the tendency; a beta plane written into m_f_vertex by a
    user kernel changes only vn's tendency."""
    out = run("term_switches")
    assert "PASS" in out, out
    assert out.count(" 1, equals the C ABI switch 1, restored 1") == 9, out


def test_cpp_model_variants():
    """The C++ LinearShallowWaterModel and the drag option against twins
    made through the C ABI: tendencies and RK4 / LSRK5 steps bitwise
    equal; an exception from an additional_tendency override reaches the
    caller with its own type and leaves the model usable."""
    out = run("model_variants")
    assert "PASS" in out and out.count("twin 1") == 2, out
    assert "hook exceptions: rethrown 1, usable after 1" in out, out


def test_cpp_aux_state_and_field_tendencies():
    """The C++ drop-in's m_aux_state and compute_h/vn/tr_tendency: after
    compute_tendency the three per-field methods reproduce it bit for bit,
    increment adds it again, m_aux_state.compute of another state gives
    that state's mean thickness exactly, and a plain model's first step
    launches the fused graph (its hook is dropped when the stepper is
    built)."""
    out = run("field_tendencies")
    assert "PASS" in out, out
    assert "bit for bit 1" in out and "again 1" in out, out


def test_rcp_nr_within_one_ulp_of_division():
    """The kernels' Newton-Raphson reciprocal (rcp.approx.ftz.f64 plus two
    Newton steps, swg_device.cuh) against CUDA's IEEE 1.0 / x on the device:
    log-spaced 1e-6 .. 1e6 of both signs, random mantissas in every binade of
    [2^-40, 2^40] and thin-layer thicknesses 1e-3 .. 1e1.  Bound: 1 ulp of the
    correctly rounded quotient (measured maximum printed)."""
    import re
    out = run("rcp_accuracy")
    m = re.search(r"samples (\d+) max_ulp (\d+)", out)
    assert m, out
    assert int(m.group(1)) > 600000
    assert int(m.group(2)) <= 1, out


def test_fp64_issue_rate_is_measured():
    """swg_fp64_issue_rate returns a positive DFMA / DADD / DMUL rate below
    the architectural ceiling of 2 FP64 thread-instructions per SM per clock
    at the GPU's maximum clock."""
    import omega_playground_gb300 as og
    import torch
    props = torch.cuda.get_device_properties(0)
    ceiling = 2.0 * props.multi_processor_count * 2.2e9
    for op in ("dfma", "dadd", "dmul"):
        rate, ms = og.fp64_issue_rate(op, 4000)
        assert 0 < rate < ceiling and ms > 0, (op, rate)
