"""Checks at the headline workload's full size (512^2 cells x 64^2 velocities
on [-6, 6]^2, UGKS + BGK, Kn = 1e-3, extrapolation boundaries, FP32 split
form): the oracle cannot run at that size, so these use properties that hold
at any size.

- A uniform Maxwellian is a fixed point of the step: every face of a
  direction sees the same states, its face moments are bit-identical to its
  neighbours', so w must come back bit-identical and the residual exactly 0.
- The step commutes with the mirror x -> 1 - x, u -> -u: from a state that
  is mirror-symmetric (rho, V, lambda even and U odd about x = 1/2), rho, V,
  lambda stay even and U odd, to FP32 rounding.  Every pass-A segment, pass-B
  strip and TMA box of the full grid takes part, so an offset or halo error
  anywhere in the grid breaks the symmetry.  This check uses midpoint
  velocity weights: the composite Newton-Cotes weights of 64 points are not
  symmetric under u -> -u (63 intervals are not a multiple of 4), so with
  them the reference algorithm itself is only symmetric to quadrature error.

Both run with the launch shapes the autotuner picks for this workload
(4-column strips, two velocities per thread, 64 rows, 2 faces per warp) and
with the untuned defaults (one velocity per thread).
"""
import numpy as np
import pytest

import kitgpu
from kitgpu.setup import prim_conserve
from kitgpu.solver import Handle, kb_config

pytestmark = pytest.mark.gpu

NX = NY = 512
NV = 64


SHAPES = [(4, 64, 64, 2), (0, 0, 0, 0), (4, 64, 64, 8)]  # march_tx, march_ry, march_bs, mom_ts


def headline_cfg(vmesh="newton"):
    return dict(matter="gas", case="quadrant", space="2d2f2v", flux="ugks", collision="bgk",
                nSpecies=1, interpOrder=2, limiter="vanleer", boundary="extra", cfl=0.5,
                maxTime=1.0, x0=0.0, x1=1.0, nx=NX, nxg=1, y0=0.0, y1=1.0, ny=NY, nyg=1,
                umin=-6.0, umax=6.0, nu=NV, vmin=-6.0, vmax=6.0, nv=NV, vMeshType=vmesh,
                knudsen=1e-3, mach=0.0, prandtl=2.0 / 3.0, inK=1.0, omega=0.81, alphaRef=1.0,
                omegaRef=0.5)


def headline_handle(shape, vmesh="newton"):
    KS = kitgpu.solver_set(headline_cfg(vmesh))
    vs = KS.vs
    h = Handle(kb_config(KS, "fp32"), vs.flat(vs.u), vs.flat(vs.v), vs.flat(vs.weights))
    h.set_tuning(*shape)
    return KS, h


def cells_w(prim, gamma):
    """w of every cell from prim [ncell, 4] (prim_conserve, vectorised)."""
    rho, U, V, lam = prim.T
    E = 0.5 * rho / lam / (gamma - 1.0) + 0.5 * rho * (U * U + V * V)
    return np.stack([rho, rho * U, rho * V, E], axis=1)


@pytest.mark.parametrize("shape", SHAPES, ids=["tuned", "default", "ring-pass-a"])
def test_headline_size_uniform_equilibrium_is_a_fixed_point(gpu_lib, shape):
    KS, h = headline_handle(shape)
    try:
        p0 = np.array([1.0, 0.1, -0.05, 1.0])
        w0 = prim_conserve(p0, KS.gas.gamma)
        P = np.tile(p0, (h.ncell, 1))
        W = np.tile(w0, (h.ncell, 1))
        h.init_equilibrium(W, P)
        dt = h.timestep(KS.set.cfl, 0.0, 1e9)
        res = h.step(dt, 3)
        out = h.download(("w",))
        assert np.array_equal(out["w"], W)
        assert np.all(res == 0.0)
    finally:
        h.close()


@pytest.mark.parametrize("shape", SHAPES, ids=["tuned", "default", "ring-pass-a"])
def test_headline_size_mirror_symmetry(gpu_lib, shape):
    KS, h = headline_handle(shape, vmesh="rectangle")
    try:
        nxt, nyt = NX + 2, NY + 2
        x = (np.arange(nxt) - 1 + 0.5) / NX  # cell centres incl. the ghost layer
        y = (np.arange(nyt) - 1 + 0.5) / NY
        X, Y = np.meshgrid(x, y)  # [j][i]: x fastest, as the cells are stored
        c, s = np.cos(2 * np.pi * (X - 0.5)), np.sin(2 * np.pi * (X - 0.5))
        P = np.stack([1.0 + 0.3 * c * (1.0 + 0.5 * Y), 0.2 * s, 0.1 * c * (Y - 0.5),
                      1.0 + 0.2 * c], axis=-1).reshape(-1, 4)
        h.init_equilibrium(cells_w(P, KS.gas.gamma), P)
        dt = h.timestep(KS.set.cfl, 0.0, 1e9)
        h.step(dt, 5)
        p = h.download(("prim",))["prim"].reshape(nyt, nxt, 4)[1:-1, 1:-1]
        m = p[:, ::-1]  # the mirror image x -> 1 - x
        # the state moved (the check is not vacuous) ...
        assert np.max(np.abs(p[..., 0] - P.reshape(nyt, nxt, 4)[1:-1, 1:-1, 0])) > 1e-4
        # ... and stayed symmetric: rho, V, lambda even, U odd (U against the
        # thermal speed 1 / sqrt(lambda)), to FP32 rounding
        tol = 1e-5
        assert np.max(np.abs(p[..., 0] - m[..., 0]) / p[..., 0]) < tol
        assert np.max(np.abs(p[..., 3] - m[..., 3]) / p[..., 3]) < tol
        assert np.max(np.abs(p[..., 1] + m[..., 1]) * np.sqrt(p[..., 3])) < tol
        assert np.max(np.abs(p[..., 2] - m[..., 2]) * np.sqrt(p[..., 3])) < tol
    finally:
        h.close()
