"""Seeded synthetic workloads of the shallow-water path.

The reference benchmarks a double-vortex case (benchmark/benchmark.cpp:83-182)
and publishes no dataset; these workloads are seeded synthetic stand-ins with
the shapes, sizes and value ranges of the benchmark configurations:

  "rk4_64x64"    64x64 cells, dc 10 km, 64 levels, 1 tracer, RK4, 10 steps,
                 dt from a 0.2 gravity-wave CFL, f0 1e-4, g 9.81,
                 del2 viscosity 1e3
  "lsrk5_512x512" 512x512 cells, 64 levels, 8 tracers, 5-stage LSRK,
                 100 steps, viscosity del2 1e3 / del4 1e9, tracer
                 diffusion del2 1e3 / del4 1e9, plus geostrophic velocity
                 noise (rms 0.05 m/s)

Initial state (per level k, so levels differ):
  h  = 1000 m + two Gaussian bumps (amplitude 1 m, e-folding width 0.1 Lx,
       periodic minimum-image distance), centres drawn from the seed;
  vn = 0, or -(psi(v1) - psi(v0)) / dv of a random vertex streamfunction
       (divergence-free), scaled to the requested rms;
  tr = h * c (thickness-weighted, like the reference's tracer state) with
       c a seeded sum of four plane sines of wavenumber <= 2 rescaled to
       [0, 1], blended across levels.
Random numbers come from a counter-based SplitMix64, so the arrays are the
same on every machine for a given seed.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)


def splitmix64(seed: int, counter: np.ndarray) -> np.ndarray:
    """SplitMix64 output for stream `seed` at positions `counter` (uint64)."""
    with np.errstate(over="ignore"):
        z = (np.uint64(seed) * _GOLDEN + (counter.astype(np.uint64)
                                          + np.uint64(1)) * _GOLDEN)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, n: int, offset: int = 0) -> np.ndarray:
    """n doubles in [0, 1) (53 random bits each)."""
    c = np.arange(offset, offset + n, dtype=np.uint64)
    return (splitmix64(seed, c) >> np.uint64(11)).astype(np.float64) * 2.0**-53


@dataclasses.dataclass(frozen=True)
class Workload:
    name: str
    nx: int
    ny: int
    dc: float
    nlayers: int
    ntracers: int
    stepper: str          # "rk4" or "lsrk"
    nstages: int          # stages per step (4 for RK4)
    nsteps: int
    f0: float = 1e-4
    grav: float = 9.81
    visc_del2: float = 0.0
    visc_del4: float = 0.0
    eddy_diff2: float = 0.0
    eddy_diff4: float = 0.0
    vn_noise_rms: float = 0.0
    h0: float = 1000.0
    seed: int = 20240601
    cfl: float = 0.2

    @property
    def dt(self) -> float:
        return self.cfl * self.dc / math.sqrt(self.grav * self.h0)

    @property
    def ncells(self) -> int:
        return self.nx * self.ny

    def params(self):
        from .shallow_water import ShallowWaterParams
        return ShallowWaterParams(m_f0=self.f0, m_grav=self.grav,
                                  m_visc_del2=self.visc_del2,
                                  m_visc_del4=self.visc_del4,
                                  m_eddy_diff2=self.eddy_diff2,
                                  m_eddy_diff4=self.eddy_diff4,
                                  m_ntracers=self.ntracers)

    def param_kwargs(self) -> dict:
        return dict(f0=self.f0, grav=self.grav, visc_del2=self.visc_del2,
                    visc_del4=self.visc_del4, eddy_diff2=self.eddy_diff2,
                    eddy_diff4=self.eddy_diff4, ntracers=self.ntracers)

    def cell_level_stages(self, nsteps: int | None = None) -> int:
        n = self.nsteps if nsteps is None else nsteps
        return self.ncells * self.nlayers * self.nstages * n

    def alg_bytes_per_stage(self) -> int:
        """Algorithmic HBM bytes of one stage: 8-byte words x (1 h + 3 vn +
        T tracers) per cell-level x 4 unavoidable accesses (read state,
        read tendency/accumulator, write both)."""
        return 32 * (4 + self.ntracers) * self.ncells * self.nlayers

    def scaled(self, **kw) -> "Workload":
        return dataclasses.replace(self, **kw)


WORKLOADS = {
    "rk4_64x64": Workload("rk4_64x64", 64, 64, 1e4, 64, 1, "rk4", 4, 10,
                          visc_del2=1e3),
    "lsrk5_512x512": Workload("lsrk5_512x512", 512, 512, 1e4, 64, 8, "lsrk",
                              5, 100, visc_del2=1e3, visc_del4=1e9,
                              eddy_diff2=1e3, eddy_diff4=1e9,
                              vn_noise_rms=0.05),
    # checkpointed adjoint: 128x128 cells, 32 levels, 2 tracers, RK4,
    # 1000 steps, 32 snapshots (the 64x64 workload's physics)
    "rk4_128x128_adjoint": Workload("rk4_128x128_adjoint", 128, 128, 1e4, 32,
                                    2, "rk4", 4, 1000, visc_del2=1e3),
}
ADJOINT_SNAPSHOTS = 32


def region_cells(mesh, seed: int, frac: float = 0.25) -> np.ndarray:
    """Cells inside a seeded axis-aligned rectangle covering `frac` of each
    periodic dimension (the loss's target region)."""
    Lx, Ly = mesh.m_period_x, mesh.m_period_y
    u = uniform(seed, 2)
    x0, y0 = u[0] * Lx * (1 - frac), u[1] * Ly * (1 - frac)
    xc, yc = np.asarray(mesh.m_x_cell), np.asarray(mesh.m_y_cell)
    inside = ((xc >= x0) & (xc < x0 + frac * Lx) &
              (yc >= y0) & (yc < y0 + frac * Ly))
    return np.nonzero(inside)[0]


def loss_and_grad(h, vn, tr, region, h_ref: float = 1000.0):
    """L = sum over region cells and levels of (h - h_ref)^2, plus for every
    tracer and level the variance over the region of the concentration
    tr / h.  Returns L and (dL/dh, dL/dvn, dL/dtr)."""
    hr = h[region]                                   # [R][K]
    L = float(np.sum((hr - h_ref) ** 2))
    gh = np.zeros_like(h)
    gh[region] = 2.0 * (hr - h_ref)
    gtr = np.zeros_like(tr)
    R = len(region)
    for l in range(tr.shape[0]):
        n = tr[l][region] / hr                       # [R][K]
        dev = n - n.mean(axis=0, keepdims=True)
        L += float(np.sum(dev * dev) / R)
        g = 2.0 * dev / R                            # dL/dn
        gtr[l][region] = g / hr
        gh[region] -= g * n / hr
    return L, (gh, np.zeros_like(vn), gtr)


def lognormal_visc(ncells: int, seed: int, median: float = 1e3,
                   sigma: float = 0.5) -> np.ndarray:
    """Per-cell del2 viscosity, log-normal around `median` (Box-Muller on
    SplitMix64 uniforms)."""
    u = uniform(seed, 2 * ncells)
    z = np.sqrt(-2.0 * np.log(u[:ncells] + 2.0**-60)) * \
        np.cos(2 * np.pi * u[ncells:])
    return median * np.exp(sigma * z)


def visc_scaling(mesh, visc_cell: np.ndarray, visc_del2: float) -> np.ndarray:
    """mesh_scaling_del2 realising a per-cell viscosity on edges:
    visc_e = (visc_c0 + visc_c1) / 2 = visc_del2 * scale_e."""
    coe = np.asarray(mesh.m_cells_on_edge if hasattr(mesh, "m_cells_on_edge")
                     else mesh.tables["cells_on_edge"])
    return 0.5 * (visc_cell[coe[:, 0]] + visc_cell[coe[:, 1]]) / visc_del2


ADJOINT_ENSEMBLE_NX = (32, 64, 96, 128)


def adjoint_ensemble(n: int = 32, seed: int = 20240603,
                     nx_choices=ADJOINT_ENSEMBLE_NX, levels=(16, 64),
                     nsteps: int = 300):
    """Members of the batched adjoint: nx from `nx_choices`, levels uniform in
    `levels`, 2 tracers, RK4, `nsteps` steps, del2 viscosity realised as a
    per-cell log-normal field (see lognormal_visc)."""
    r = uniform(seed, 2 * n).reshape(n, 2)
    base = WORKLOADS["rk4_128x128_adjoint"]
    out = []
    for i in range(n):
        nx = nx_choices[int(r[i, 0] * len(nx_choices))]
        K = levels[0] + int(r[i, 1] * (levels[1] - levels[0] + 1))
        out.append(base.scaled(name=f"adjmember{i}", nx=nx, ny=nx, nlayers=K,
                               nsteps=nsteps, seed=seed + 1000 * i))
    return out


ENSEMBLE_NX = (32, 48, 64, 96, 128, 192)


def ensemble(n: int = 64, seed: int = 20240602, nx_choices=ENSEMBLE_NX,
             levels=(16, 96), tracers=(1, 4), nsteps: int = 200):
    """Members of the batched ensemble: nx drawn from `nx_choices`, level
    count uniform in `levels`, tracer count uniform in `tracers`, RK4, the
    64x64 workload's physics (del2 viscosity 1e3), each with its own seed."""
    r = uniform(seed, 3 * n).reshape(n, 3)
    base = WORKLOADS["rk4_64x64"]
    out = []
    for i in range(n):
        nx = nx_choices[int(r[i, 0] * len(nx_choices))]
        K = levels[0] + int(r[i, 1] * (levels[1] - levels[0] + 1))
        T = tracers[0] + int(r[i, 2] * (tracers[1] - tracers[0] + 1))
        out.append(base.scaled(name=f"member{i}", nx=nx, ny=nx, nlayers=K,
                               ntracers=T, nsteps=nsteps, seed=seed + 1000 * i))
    return out


def _min_image(d: np.ndarray, L: float) -> np.ndarray:
    return d - L * np.round(d / L)


def initial_state(mesh, wl: Workload):
    """(h [C][K], vn [E][K], tr [T][C][K]) for `wl` on `mesh` (any object
    with the planar-hex tables as m_x_cell, m_y_cell, m_cells_on_edge ...)."""
    K, T, C = wl.nlayers, wl.ntracers, wl.nx * wl.ny
    Lx, Ly = mesh.m_period_x, mesh.m_period_y
    xc, yc = np.asarray(mesh.m_x_cell), np.asarray(mesh.m_y_cell)
    width = 0.1 * Lx
    # two bump centres per level
    u = uniform(wl.seed, 4 * K).reshape(K, 2, 2)
    h = np.full((C, K), wl.h0)
    for b in range(2):
        cx, cy = u[:, b, 0] * Lx, u[:, b, 1] * Ly          # [K]
        dx = _min_image(xc[:, None] - cx[None, :], Lx)
        dy = _min_image(yc[:, None] - cy[None, :], Ly)
        h += np.exp(-(dx * dx + dy * dy) / (width * width))
    # velocity
    E = 3 * C
    vn = np.zeros((E, K))
    if wl.vn_noise_rms > 0:
        V = 2 * C
        psi = uniform(wl.seed + 1, V * K).reshape(V, K) - 0.5
        voe = np.asarray(mesh.m_vertices_on_edge)
        dv = np.asarray(mesh.m_dv_edge)
        vn = -(psi[voe[:, 1]] - psi[voe[:, 0]]) / dv[:, None]
        rms = np.sqrt(np.mean(vn * vn, axis=0))
        vn *= (wl.vn_noise_rms / rms)[None, :]
    # tracers: per-tracer sum of four plane sines, blended across levels
    tr = np.zeros((T, C, K))
    if T:
        base = np.empty((T, C))
        for l in range(T):
            r = uniform(wl.seed + 2 + l, 16)
            c = np.zeros(C)
            for m in range(4):
                kx = int(r[4 * m] * 5) - 2
                ky = int(r[4 * m + 1] * 5) - 2
                if kx == 0 and ky == 0:
                    kx = 1
                amp = 0.5 + 0.5 * r[4 * m + 2]
                ph = 2 * math.pi * r[4 * m + 3]
                c += amp * np.sin(2 * math.pi * (kx * xc / Lx + ky * yc / Ly)
                                  + ph)
            span = c.max() - c.min()
            # a one-cell mesh has no spread to rescale: uniform 1/2
            base[l] = (c - c.min()) / span if span > 0 else 0.5
        alpha = 0.5 * np.arange(K) / max(K - 1, 1)            # [K]
        for l in range(T):
            nxt = base[(l + 1) % T]
            cl = base[l][:, None] * (1 - alpha)[None, :] + \
                nxt[:, None] * alpha[None, :]
            tr[l] = h * cl
    return h, vn, tr
