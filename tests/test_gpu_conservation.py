"""Conservation of the FP32-split form on the GPU.

The split form keeps the conservative update in FP64: w += (fw_in - fw_out) / ds
with fw summed from FP32 distributions into compensated FP64 face moments
(step!, src/Solver/step_2f.jl:6-64, :179-249).  Every interior face flux is
added to one cell and subtracted from its neighbour, so the totals change only
by what crosses the boundary, up to the FP64 round-off of the per-cell
additions.

- Mass in a closed box of Maxwell diffuse walls: the wall density is chosen so
  no mass crosses a wall (flux_boundary_maxwell!, src/Flux/flux_boundary.jl:39-61,
  :190-220), so total mass is constant to FP64 round-off, here over 200 steps
  of a lid-driven cavity and of a Sod tube between two walls.
- Mass, momentum and energy: walls exchange momentum and heat, so the change
  of each total over one step must equal what the boundary faces carried in
  (their fw, downloaded after evolve!), again to FP64 round-off.

Bound: relative change (or imbalance) <= 1e-13 of the total.
"""
import ctypes

import numpy as np
import pytest

import kitgpu
from kitgpu import _native as N
from cases import cavity, sod

pytestmark = pytest.mark.gpu

TOL = 1e-13


def _totals(KS, ctr):
    """Sum over physical cells of w times the cell volume."""
    hd = ctr.handle
    c = hd.cfg
    w = hd.download(("w",))["w"]
    if KS.dim == 1:
        return w[c.ngx:c.ngx + c.nx].sum(axis=0) * (c.x1 - c.x0) / c.nx
    grid = w.reshape(hd.nyt, hd.nxt, -1)[c.ngy:c.ngy + c.ny, c.ngx:c.ngx + c.nx]
    return grid.reshape(-1, hd.nw).sum(axis=0) * (c.x1 - c.x0) / c.nx * (c.y1 - c.y0) / c.ny


def _face_fw(ctr):
    hd = ctr.handle
    fw = np.zeros((hd.nface, hd.nw))
    N.check(hd.lib.kb_download_faces(hd.h, ctypes.c_double(0.0), N.ptr(fw), None, None))
    return fw


def _boundary_inflow(KS, ctr, fw):
    """Net amount carried into the domain through the boundary faces in one
    step (fw holds the time-integrated flux times the face length)."""
    c = ctr.handle.cfg
    if KS.dim == 1:
        return fw[0] - fw[c.nx]
    nfx = (c.nx + 1) * c.ny
    fx = fw[:nfx].reshape(c.ny, c.nx + 1, -1)
    fy = fw[nfx:].reshape(c.ny + 1, c.nx, -1)
    return fx[:, 0].sum(axis=0) - fx[:, c.nx].sum(axis=0) + fy[0].sum(axis=0) - fy[c.ny].sum(axis=0)


CLOSED = [
    ("cavity-kcu-shakhov-lid", cavity(nx=32, ny=32, nu=28, nv=28)),
    ("cavity-ugks-bgk-lid", cavity(nx=24, ny=20, nu=24, nv=24, flux="ugks", coll="bgk", Kn=0.01)),
    ("sod-kfvs-shakhov-walls", sod(nx=100, nu=64, flux="kfvs", coll="shakhov", bc="maxwell")),
]


@pytest.mark.parametrize("name,cfg", CLOSED, ids=[c[0] for c in CLOSED])
def test_fp32_closed_box_mass(gpu_lib, name, cfg):
    KS, ctr, *faces, t = kitgpu.initialize(cfg, precision="fp32")
    dt = kitgpu.timestep(KS, ctr, 0.0)
    m0 = _totals(KS, ctr)[0]
    kitgpu.step(KS, ctr, dt, 200)
    m1 = _totals(KS, ctr)[0]
    assert abs(m1 - m0) <= TOL * abs(m0), (m0, m1, (m1 - m0) / m0)


@pytest.mark.parametrize("name,cfg", CLOSED, ids=[c[0] for c in CLOSED])
def test_fp32_boundary_balance(gpu_lib, name, cfg):
    """Change of mass, momentum and energy over a step = boundary inflow."""
    KS, ctr, *faces, t = kitgpu.initialize(cfg, precision="fp32")
    dt = kitgpu.timestep(KS, ctr, 0.0)
    kitgpu.step(KS, ctr, dt, 30)
    scale = np.abs(_totals(KS, ctr))
    scale[1:KS.dim + 1] = scale[0]  # momentum against the mass scale (it starts near 0)
    for _ in range(5):
        w0 = _totals(KS, ctr)
        kitgpu.reconstruct(KS, ctr)
        kitgpu.evolve(KS, ctr, *faces, dt)
        inflow = _boundary_inflow(KS, ctr, _face_fw(ctr))
        r = np.zeros(KS.dim + 2)
        kitgpu.update(KS, ctr, *faces, dt, r)
        w1 = _totals(KS, ctr)
        err = np.abs((w1 - w0) - inflow) / scale
        assert np.all(err <= TOL), err
