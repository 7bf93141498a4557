"""Index arithmetic at the largest meshes the library takes.

swg_mesh_create accepts meshes whose edge·level and (vertex + cell)·level
counts stay below 2^31.  A 1024x1024-cell mesh with 640 levels puts both at
2,013,265,920 (94 % of the limit).  Every tendency term works on one level at
a time, so after one LSRK5 step the lowest and the highest 8 levels of that
state must equal, bit for bit, an 8-level model stepped from the same
levels.  The fields are written and compared on the device through
zero-copy torch views, so the host holds no 640-level array.  The model
(del2 viscosity, no tracers) needs about 155 GB of device memory."""
import math

import numpy as np
import pytest

import omega_playground_gb300 as og

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

NX = NY = 1024
K_BIG, K_SMALL = 640, 8
DC = 1e4


def set_fields(mesh, S, K, k_offset=0):
    """Smooth h and vn, level-dependent phases, on the device."""
    dev = torch.device("cuda")
    xc = torch.from_numpy(np.asarray(mesh.m_x_cell)).to(dev)[:, None]
    yc = torch.from_numpy(np.asarray(mesh.m_y_cell)).to(dev)[:, None]
    xe = torch.from_numpy(np.asarray(mesh.m_x_edge)).to(dev)[:, None]
    ye = torch.from_numpy(np.asarray(mesh.m_y_edge)).to(dev)[:, None]
    ang = torch.from_numpy(np.asarray(mesh.m_angle_edge)).to(dev)[:, None]
    Lx, Ly = mesh.m_period_x, mesh.m_period_y
    h, vn, _ = S.as_tensors()
    for k1 in range(0, K, 64):  # level blocks keep the temporaries small
        k2 = min(K, k1 + 64)
        kk = torch.arange(k_offset + k1, k_offset + k2, device=dev,
                          dtype=torch.float64)[None, :]
        h[:, k1:k2] = (1000.0 + 2.0 * torch.sin(2 * math.pi * xc / Lx +
                                                0.01 * kk)
                       * torch.cos(2 * math.pi * yc / Ly))
        ux = 0.3 * torch.cos(2 * math.pi * ye / Ly + 0.02 * kk)
        uy = 0.2 * torch.sin(2 * math.pi * xe / Lx - 0.01 * kk)
        vn[:, k1:k2] = torch.cos(ang) * ux + torch.sin(ang) * uy
    torch.cuda.synchronize()


@pytest.mark.skipif(not torch.cuda.is_available() or
                    torch.cuda.get_device_properties(0).total_memory < 200e9,
                    reason="needs a GPU with >= 200 GB")
def test_levels_of_a_mesh_at_the_index_limit_match_a_small_model():
    params = og.ShallowWaterParams(m_f0=1e-4, m_grav=9.81, m_visc_del2=1e3)
    big = og.PlanarHexagonalMesh(NX, NY, DC, K_BIG)
    E, V, C = big.m_nedges, big.m_nvertices, big.m_ncells
    assert E * K_BIG == (V + C) * K_BIG == 2013265920 < 2**31
    small = og.PlanarHexagonalMesh(NX, NY, DC, K_SMALL)
    m_small = og.ShallowWaterModel(small, params)
    dt = 0.2 * DC / math.sqrt(9.81 * 1000.0)
    outs = {}
    for k0 in (0, K_BIG - K_SMALL):
        S = og.ShallowWaterState(small, params)
        set_fields(small, S, K_SMALL, k0)
        before = tuple(t.clone() for t in S.as_tensors()[:2])
        og.LSRKStepper(m_small, 5).step(S, 0.0, dt, 1)
        outs[k0] = tuple(t.clone() for t in S.as_tensors()[:2])
        assert not torch.equal(outs[k0][1], before[1])  # the step moved vn
        del S
    m_big = og.ShallowWaterModel(big, params)
    B = og.ShallowWaterState(big, params)
    set_fields(big, B, K_BIG)
    torch.cuda.empty_cache()
    og.LSRKStepper(m_big, 5).step(B, 0.0, dt, 1)
    torch.cuda.synchronize()
    h, vn, _ = B.as_tensors()
    for k0, (hs, vs) in outs.items():
        assert torch.isfinite(hs).all() and torch.isfinite(vs).all()
        assert torch.equal(h[:, k0:k0 + K_SMALL], hs), k0
        assert torch.equal(vn[:, k0:k0 + K_SMALL], vs), k0
