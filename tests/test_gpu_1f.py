"""The 1F models, 1D1F1V and 2D1F2V, through the C ABI against the FP64
oracle's own 1F restatement (flux_kfvs! 1F1V / 1F2V, src/Flux/flux_kfvs.jl:238-262,
:615-650; flux_kcu! 1D1F1V / 2D1F2V, src/Flux/flux_kcu.jl:241-303, :828-894;
step! src/Solver/step_1f.jl:6-58, :164-224; the 2D1F2V Maxwell wall,
src/Flux/flux_boundary.jl:158-186).

The device runs a 1F solve as the 2F step with the second distribution
absent (b held at zero, its equilibrium B = 0 and the Shakhov factor
2 lambda c^2 - 5): the plain FP64 form must match the oracle within 1e-12 in
rho, U, T and f, the FP32-split form within 1e-5, and b must stay exactly 0.
The first cases follow the reference's own 1F test configurations
(test/config_1d1f1v.txt: shock, KFVS + BGK, inK = 0, Pr = 1, 50 cells with 2
ghost layers, 24 velocities on [-12, 12]; test/config_2d1f.txt: cavity,
KFVS + BGK, Maxwell walls, 21^2 cells with a ghost layer, 16^2 velocities).
"""
import numpy as np
import pytest

import kitgpu
from cases import cavity, oracle_for, quadrant, rel, rho_u_t_error, shock, sod

pytestmark = pytest.mark.gpu


def one_f(cfg, **kw):
    c = dict(cfg, inK=0.0, **kw)
    c["space"] = "1d1f1v" if cfg["space"].startswith("1d") else "2d1f2v"
    return c


CASES = [
    ("shock-kfvs-bgk-config_1d1f1v", one_f(shock(nx=50, nu=24, Ma=2.0, flux="kfvs", coll="bgk",
                                                 ng=2), umin=-12.0, umax=12.0, prandtl=1.0), 25),
    ("sod-kfvs-bgk", one_f(sod(flux="kfvs", coll="bgk")), 25),
    ("sod-kfvs-shakhov", one_f(sod(flux="kfvs", coll="shakhov")), 25),
    ("sod-kcu-bgk-extra", one_f(sod(flux="kcu", coll="bgk", bc="extra", ng=1)), 25),
    ("sod-kcu-shakhov", one_f(sod(flux="kcu", coll="shakhov", Kn=1e-2)), 25),
    ("cavity-kfvs-bgk-config_2d1f", one_f(cavity(nx=21, ny=21, nu=16, nv=16, flux="kfvs",
                                                 coll="bgk", ng=1, vmesh="rectangle", Kn=1.0),
                                          prandtl=1.0), 8),
    ("cavity-kcu-bgk", one_f(cavity(nx=12, ny=10, nu=12, nv=14, coll="bgk")), 8),
    ("quadrant-kfvs-bgk-extra", one_f(quadrant(nx=14, ny=13, nu=12, nv=12, flux="kfvs")), 8),
    ("quadrant-kcu-bgk-extra", one_f(quadrant(nx=17, ny=18, nu=8, nv=8, flux="kcu", Kn=1e-2)), 8),
]


def _run(cfg, n, prec):
    KS, ctr, *faces, t = kitgpu.initialize(cfg, precision=prec)
    assert KS.nf == 1 and ctr.handle.cfg.nf == 1
    orc = oracle_for(KS)
    dt = kitgpu.timestep(KS, ctr, 0.0)
    assert dt == pytest.approx(orc.timestep(KS.set.cfl, 0.0, KS.set.maxTime), rel=1e-14)
    rg = kitgpu.step(KS, ctr, dt, n)
    ro = orc.step(dt, n)
    return ctr.handle.download(), orc.get_state(), rg, ro


@pytest.mark.parametrize("name,cfg,n", CASES, ids=[c[0] for c in CASES])
def test_1f_fp64_parity(gpu_lib, name, cfg, n):
    g, o, rg, ro = _run(cfg, n, "fp64")
    w, p, f, b = o
    e = rho_u_t_error(g["prim"], p)
    assert max(e) < 1e-12, e
    assert rel(g["w"][:, 0], w[:, 0]) < 1e-12
    assert np.max(np.abs(g["h"] - f)) / np.max(np.abs(f)) < 1e-12
    assert np.all(g["b"] == 0.0)
    assert np.allclose(rg, ro, rtol=1e-9, atol=1e-300)


@pytest.mark.parametrize("name,cfg,n", CASES, ids=[c[0] for c in CASES])
def test_1f_fp32_split(gpu_lib, name, cfg, n):
    g, o, rg, ro = _run(cfg, 4 * n, "fp32")
    e = rho_u_t_error(g["prim"], o[1])
    assert max(e) < 1e-5, e
    assert np.all(g["b"] == 0.0)


def test_1f_gamma_from_inK(gpu_lib):
    """heat_capacity_ratio(inK, D) for 1F spaces (src/Struct/struct_property.jl:476-492):
    gamma = 3 in 1D1F1V and 2 in 2D1F2V with inK = 0."""
    KS1 = kitgpu.solver_set(CASES[1][1])
    KS2 = kitgpu.solver_set(CASES[5][1])
    assert KS1.gas.gamma == 3.0 and KS2.gas.gamma == 2.0
