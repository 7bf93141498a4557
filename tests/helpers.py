"""Shared helpers of the test suite: golden fixtures, oracle runs and the
normwise relative difference used by every parity bound."""
from __future__ import annotations

import glob
import os

import numpy as np

import pyoracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STEPPER_KIND = {1: ("rk4", 4), 2: ("lsrk", 5), 3: ("lsrk", 1)}


def golden_names():
    return sorted(os.path.basename(f)[:-4]
                  for f in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name):
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    pi, pd = g["params_i"], g["params_d"]
    g["cfg"] = dict(nx=int(pi[0]), ny=int(pi[1]), K=int(pi[2]), T=int(pi[3]),
                    stepper=int(pi[4]), nsteps=int(pi[5]),
                    disable_h=bool(pi[6]), disable_vn=bool(pi[7]),
                    dc=float(pd[0]), f0=float(pd[1]), grav=float(pd[2]),
                    visc_del2=float(pd[3]), visc_del4=float(pd[4]),
                    eddy_diff2=float(pd[5]), eddy_diff4=float(pd[6]),
                    dt=float(pd[7]), t0=float(pd[8]))
    return g


def oracle_model(cfg):
    m = pyoracle.OracleMesh(cfg["nx"], cfg["ny"], cfg["dc"], cfg["K"])
    md = pyoracle.OracleModel(
        m, f0=cfg["f0"], grav=cfg["grav"], visc_del2=cfg["visc_del2"],
        visc_del4=cfg["visc_del4"], eddy_diff2=cfg["eddy_diff2"],
        eddy_diff4=cfg["eddy_diff4"], ntracers=cfg["T"],
        disable_h_tendency=cfg["disable_h"],
        disable_vn_tendency=cfg["disable_vn"])
    return m, md


def rel_diff(a, b):
    """max |a - b| / max |b| (normwise relative, L-infinity); 0 for empty."""
    a, b = np.asarray(a), np.asarray(b)
    if b.size == 0:
        return 0.0
    scale = np.max(np.abs(b))
    if scale == 0:
        return float(np.max(np.abs(a)))
    return float(np.max(np.abs(a - b)) / scale)
