"""Generate the golden fixtures in this directory from the reference itself.

Each scenario is run through ``oracle/_ref/ref_driver``: the omega_playground
reference's own, unmodified ``src/`` sources compiled with g++ against the
host-only Kokkos shim (``oracle/Makefile``, target ``ref``).  The inputs (seeded
here) and every output (mesh tables, auxiliary fields and tendency of one
``compute_tendency``, diagnostics, state after N steps) are stored together in
``<scenario>.npz``, so the fixtures stand on their own.

The reference's six CTest programs, built the same way, are run too and
their printed error/rate tables are saved in ``reference_tests.txt``.

Needs the reference checkout (default /root/reference, or $OMEGA_REFERENCE);
run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle  # noqa: E402

STEPPERS = {"none": 0, "rk4": 1, "lsrk5": 2, "lsrk1": 3}

# name: nx, ny, dc, K, T, stepper, nsteps, dt, params, seed
SCENARIOS = {
    # every term on, RK4
    "rk4_all_terms": dict(nx=8, ny=8, dc=1e4, K=3, T=2, stepper="rk4",
                          nsteps=3, dt=20.0, f0=1e-4, grav=9.81,
                          visc_del2=1e3, visc_del4=1e9, eddy_diff2=1e3,
                          eddy_diff4=1e9, seed=11),
    # every term on, 5-stage LSRK, rectangular mesh
    "lsrk5_all_terms": dict(nx=6, ny=10, dc=2e4, K=2, T=1, stepper="lsrk5",
                            nsteps=2, dt=30.0, f0=1e-4, grav=9.81,
                            visc_del2=5e2, visc_del4=2e9, eddy_diff2=2e3,
                            eddy_diff4=5e8, seed=12),
    # forward Euler (1-stage LSRK), no dissipation, no tracers
    "lsrk1_inviscid": dict(nx=4, ny=4, dc=1e4, K=1, T=0, stepper="lsrk1",
                           nsteps=4, dt=10.0, f0=1e-4, grav=9.81, seed=13),
    # odd ny: the reference's racy mesh construction, serial last writer
    "odd_ny_rk4": dict(nx=5, ny=7, dc=1e4, K=1, T=1, stepper="rk4", nsteps=2,
                       dt=15.0, f0=6e-5, grav=9.80616, visc_del2=1e3,
                       seed=14),
    # frozen h and vn (tracer-transport configuration of the tracer tests)
    "frozen_flow_tracers": dict(nx=8, ny=6, dc=1e4, K=2, T=3,
                                stepper="lsrk5", nsteps=3, dt=25.0, f0=1e-4,
                                grav=9.81, eddy_diff2=1e3, eddy_diff4=1e9,
                                disable_h=1, disable_vn=1, seed=15),
    # the 64x64 RK4 workload's physics on a 16x16 mesh, 10 steps
    "rk4_10_steps": dict(nx=16, ny=16, dc=1e4, K=4, T=1, stepper="rk4",
                         nsteps=10, dt=20.19, f0=1e-4, grav=9.81,
                         visc_del2=1e3, seed=16),
    # the smallest meshes: one column of cells (each cell its own east and
    # west neighbour) and an odd 2x3 mesh, every term on
    "tiny_1x2_lsrk5": dict(nx=1, ny=2, dc=1e4, K=2, T=1, stepper="lsrk5",
                           nsteps=3, dt=20.0, f0=1e-4, grav=9.81,
                           visc_del2=1e3, visc_del4=1e9, eddy_diff2=1e3,
                           eddy_diff4=1e9, seed=18),
    "tiny_2x3_rk4": dict(nx=2, ny=3, dc=1e4, K=3, T=2, stepper="rk4",
                         nsteps=3, dt=20.0, f0=1e-4, grav=9.81,
                         visc_del2=1e3, visc_del4=1e9, eddy_diff2=1e3,
                         eddy_diff4=1e9, seed=19),
    # one field frozen: h (RK4 stage inputs keep the step's h) and vn
    "frozen_h_rk4": dict(nx=8, ny=6, dc=1e4, K=3, T=2, stepper="rk4",
                         nsteps=3, dt=20.0, f0=1e-4, grav=9.81,
                         visc_del2=1e3, visc_del4=1e9, eddy_diff2=1e3,
                         eddy_diff4=1e9, disable_h=1, seed=20),
    "frozen_vn_lsrk5": dict(nx=6, ny=8, dc=1e4, K=2, T=2, stepper="lsrk5",
                            nsteps=3, dt=20.0, f0=1e-4, grav=9.81,
                            visc_del2=1e3, visc_del4=1e9, eddy_diff2=1e3,
                            eddy_diff4=1e9, disable_vn=1, seed=21),
    # every term on, 5-stage LSRK, 1000 steps (long-run agreement)
    "lsrk5_1000_steps": dict(nx=12, ny=10, dc=1e4, K=3, T=2, stepper="lsrk5",
                             nsteps=1000, dt=20.0, f0=1e-4, grav=9.81,
                             visc_del2=1e3, visc_del4=1e9, eddy_diff2=1e3,
                             eddy_diff4=1e9, seed=17),
}


def make_inputs(sc: dict) -> dict:
    rng = np.random.default_rng(sc["seed"])
    nx, ny, K, T = sc["nx"], sc["ny"], sc["K"], sc["T"]
    m = pyoracle.OracleMesh(nx, ny, sc["dc"], K)
    Lx, Ly = m.period_x, m.period_y
    xc, yc = m.x_cell[:, None], m.y_cell[:, None]
    xe, ye = m.x_edge[:, None], m.y_edge[:, None]
    ang = m.angle_edge[:, None]
    kk = np.arange(K)[None, :]
    h = (1000.0 + 2.0 * np.sin(2 * np.pi * xc / Lx + 0.3 * kk)
         * np.cos(2 * np.pi * yc / Ly) + 0.05 * rng.standard_normal((m.ncells, K)))
    ux = 0.3 * np.cos(2 * np.pi * ye / Ly + 0.2 * kk)
    uy = 0.2 * np.sin(2 * np.pi * xe / Lx - 0.1 * kk)
    vn = (np.cos(ang) * ux + np.sin(ang) * uy
          + 0.02 * rng.standard_normal((m.nedges, K)))
    c = rng.uniform(0.0, 1.0, (T, m.ncells, K))
    tr = h[None] * c
    return dict(h=h, vn=vn, tr=tr)


def run_scenario(name: str, sc: dict, workdir: str) -> dict:
    inputs = make_inputs(sc)
    params_i = np.array([sc["nx"], sc["ny"], sc["K"], sc["T"],
                         STEPPERS[sc["stepper"]], sc["nsteps"],
                         sc.get("disable_h", 0), sc.get("disable_vn", 0)],
                        np.int32)
    params_d = np.array([sc["dc"], sc["f0"], sc["grav"],
                         sc.get("visc_del2", 0.0), sc.get("visc_del4", 0.0),
                         sc.get("eddy_diff2", 0.0), sc.get("eddy_diff4", 0.0),
                         sc["dt"], 0.0])
    out = pyoracle.run_ref_driver(
        dict(params_i=params_i, params_d=params_d, **inputs), workdir)
    rec = {f"in_{k}": v for k, v in inputs.items()}
    rec.update(params_i=params_i, params_d=params_d)
    rec.update(out)
    return rec


TABLES = ("nedges_on_cell", "edges_on_cell", "cells_on_cell",
          "vertices_on_cell", "kite_index_on_cell", "nedges_on_edge",
          "edges_on_edge", "cells_on_edge", "vertices_on_edge",
          "edges_on_vertex", "cells_on_vertex", "area_cell", "x_cell",
          "y_cell", "edge_sign_on_cell", "dc_edge", "dv_edge", "angle_edge",
          "x_edge", "y_edge", "weights_on_edge", "area_triangle",
          "x_vertex", "y_vertex", "kiteareas_on_vertex",
          "edge_sign_on_vertex")


def mesh_sweep(n: int = 12) -> None:
    """Pins the oracle on every mesh of nx, ny in 1..n cells: the
    reference's own tables and one tendency (every term on, 2 levels, one
    tracer) against the oracle's, bit for bit.  Writes mesh_sweep.txt."""
    pyoracle.build(with_reference=True)
    bad = []
    with tempfile.TemporaryDirectory() as wd:
        for nx in range(1, n + 1):
            for ny in range(1, n + 1):
                sc = dict(nx=nx, ny=ny, dc=1e4, K=2, T=1, stepper="none",
                          nsteps=0, dt=0.0, f0=1e-4, grav=9.81,
                          visc_del2=1e3, visc_del4=1e9, eddy_diff2=1e3,
                          eddy_diff4=1e9, seed=1000 * nx + ny)
                rec = run_scenario(f"{nx}x{ny}", sc, wd)
                om = pyoracle.OracleMesh(nx, ny, 1e4, 2)
                for k in TABLES:
                    if k in rec and not np.array_equal(rec[k], om.tables[k]):
                        bad.append(f"{nx}x{ny} {k}")
                md = pyoracle.OracleModel(om, f0=1e-4, grav=9.81,
                                          visc_del2=1e3, visc_del4=1e9,
                                          eddy_diff2=1e3, eddy_diff4=1e9,
                                          ntracers=1)
                got = md.compute_tendency(rec["in_h"], rec["in_vn"],
                                          rec["in_tr"])
                for k, g in zip(("tend_h", "tend_vn", "tend_tr"), got):
                    if not np.array_equal(g, rec[k]):
                        bad.append(f"{nx}x{ny} {k}")
    text = (f"oracle against the reference build on every mesh of nx, ny in "
            f"1..{n}: tables and one tendency (all terms, K = 2, T = 1)\n"
            + (f"mismatches: {', '.join(bad)}\n" if bad else
               f"{n * n} meshes, all bit-exact\n"))
    with open(os.path.join(HERE, "mesh_sweep.txt"), "w") as f:
        f.write(text)
    print(text, end="")


def main() -> None:
    """Regenerates every fixture and reference_tests.txt, or only the
    scenarios named on the command line (``--mesh-sweep``: the sweep of
    mesh_sweep())."""
    only = sys.argv[1:]
    if only == ["--mesh-sweep"]:
        mesh_sweep()
        return
    pyoracle.build(with_reference=True)
    with tempfile.TemporaryDirectory() as wd:
        for name, sc in SCENARIOS.items():
            if only and name not in only:
                continue
            rec = run_scenario(name, sc, wd)
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
            print(f"{name}: {len(rec)} arrays")
    if only:
        return
    lines = []
    for t in ("operator_convergence", "nonlinear_swe_convergence",
              "double_vortex", "tracer_advection_convergence",
              "tracer_diffusion_convergence",
              "tracer_hyperdiffusion_convergence"):
        exe = os.path.join(ROOT, "oracle", "_ref", t)
        r = subprocess.run([exe], capture_output=True, text=True, check=True)
        lines.append(f"=== {t}\n{r.stdout}")
    with open(os.path.join(HERE, "reference_tests.txt"), "w") as f:
        f.write("".join(lines))
    print("reference_tests.txt written")


if __name__ == "__main__":
    main()
