"""GPU parity at the sizes of the benchmark configurations, against the FP64
oracle.

- Sod 1D2F1V: 200 cells x 101 Newton-Cotes velocities on [-5, 5], KFVS +
  Shakhov (Kn 1e-4, omega 0.81, Pr 2/3), van Leer, CFL 0.5, run to t = 0.2 as
  solve! does (nt = floor(maxTime / dt) + 1 = 504 steps, src/Solver/solver_main.jl:12-76).
- Lid-driven cavity 2D2F2V: 64^2 cells x 28^2 Newton-Cotes velocities on
  [-5, 5]^2, KCU + Shakhov, Kn 0.075, Maxwell walls (lambda_w = 1), lid
  U = 0.15, 2000 steps (src/Config/cfg_cavity.jl:6-62).
- Four-quadrant physics of the headline workload (64^2 velocities on [-6, 6]^2,
  UGKS + BGK, Kn 1e-3) at 128^2 cells, 40 steps.

The oracle's inputs for Sod and the cavity come from the oracle's own
restatement of the reference setup (velocity grid, Newton-Cotes weights,
initial cells, wall states: oracle/oracle.py), not from kitgpu's host code,
so a setup bug cannot pass by being shared.  The four-quadrant state has no
reference preset (it is a seeded synthetic draw), so its cells come from
kitgpu and its velocity grid from the oracle's restatement.

Tolerances: the plain FP64 form within 1e-12 of the oracle in rho, U, T (U
against the thermal speed sqrt(1 / lambda), T = 1 / (2 lambda)); the
FP32-split form within 1e-5 in rho, U, T and, for the Shakhov heat flux q,
within 1e-4 of max |q|.
"""
import numpy as np
import pytest

import kitgpu
import oracle as O
import oracle_setup as OP
from cases import cavity, quadrant, rho_u_t_error, sod

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-5
TOLQ32 = 1e-4

C1 = sod(nx=200, nu=101, flux="kfvs", coll="shakhov", Kn=1e-4, maxTime=0.2)
C2 = cavity(nx=64, ny=64, nu=28, nv=28, flux="kcu", coll="shakhov", bc="maxwell", Kn=0.075)
C2_STEPS = 2000
C3S = quadrant(nx=128, ny=128, nu=64, nv=64, flux="ugks", coll="bgk", bc="extra", ng=1, Kn=1e-3)
C3S_STEPS = 40


def heat_flux(h, b, prim, u, v, wt):
    """q of every cell, heat_flux 2F1V / 2F2V (src/Theory/theory_moments.jl:530-531,
    :567-578): [ncell, 1] in 1D, [ncell, 2] in 2D."""
    U = prim[:, 1:2]
    cu = u[None, :] - U
    if v is None:
        q = 0.5 * (np.sum(wt * cu * cu * cu * h, axis=1) + np.sum(wt * cu * b, axis=1))
        return q[:, None]
    V = prim[:, 2:3]
    cv = v[None, :] - V
    c2 = cu * cu + cv * cv
    q1 = 0.5 * (np.sum(wt * cu * c2 * h, axis=1) + np.sum(wt * cu * b, axis=1))
    q2 = 0.5 * (np.sum(wt * cv * c2 * h, axis=1) + np.sum(wt * cv * b, axis=1))
    return np.stack([q1, q2], axis=1)


def q_error(ga, oa, u, v, wt):
    qg = heat_flux(ga["h"], ga["b"], ga["prim"], u, v, wt)
    qo = heat_flux(oa[2], oa[3], oa[1], u, v, wt)
    return float(np.max(np.abs(qg - qo)) / max(np.max(np.abs(qo)), 1e-300))


def _oracle_sod(KS):
    """Oracle for the Sod config from the oracle's own setup restatement."""
    mu = OP.mu_ref_of(1e-4, 1.0, 0.5)
    u, wt = O.vspace1d(-5.0, 5.0, 101, "newton")
    cfg = O.make_config(1, 200, 1, 0, 0, 101, 1, "kfvs", "shakhov", "fix", 2, 0.0, 1.0, 0.0, 1.0,
                        5.0, 0.0, 2.0, 5.0 / 3.0, mu, 0.81, 2.0 / 3.0)
    orc = O.Oracle(cfg, u, None, wt)
    orc.set_state(*O.sod_state(200, 0, 0.0, 1.0, u, 5.0 / 3.0, 2.0))
    return orc, u, None, wt


def _oracle_cavity(KS):
    mu = OP.mu_ref_of(0.075, 1.0, 0.5)
    u, v, wt = O.vspace2d(-5.0, 5.0, 28, -5.0, 5.0, 28, "newton")
    cfg = O.make_config(2, 64, 64, 0, 0, 28, 28, "kcu", "shakhov", "maxwell", 2, 0.0, 1.0, 0.0,
                        1.0, 5.0, 5.0, 1.0, 5.0 / 3.0, mu, 0.72, 2.0 / 3.0)
    orc = O.Oracle(cfg, u, v, wt)
    orc.set_state(*O.cavity_state(64, 64, 0, 0, u, v, 5.0 / 3.0, 1.0))
    for side, prim in enumerate(O.cavity_walls(64, 64, 0.0, 1.0, 0.0, 1.0)):
        orc.set_wall(side, prim)
    return orc, u, v, wt


def test_setup_restatements_agree():
    """Both setups give the same gas constants as the config text states:
    mu_ref = ref_vhs_vis(Kn, 1, 0.5) (src/Theory/theory_macro.jl:447-449)."""
    mu = 5 * (1 + 1) * (1 + 2) * np.sqrt(np.pi) / (4 * 1 * (5 - 2 * 0.5) * (7 - 2 * 0.5))
    assert kitgpu.kb_config(kitgpu.solver_set(C1)).mu_ref == pytest.approx(mu * 1e-4, rel=1e-15)
    assert kitgpu.kb_config(kitgpu.solver_set(C2)).mu_ref == pytest.approx(mu * 0.075, rel=1e-15)


@pytest.fixture(scope="module")
def sod_oracle():
    KS = kitgpu.solver_set(C1)
    orc, u, v, wt = _oracle_sod(KS)
    dt = orc.timestep(0.5, 0.0, 0.2)
    nt = int(np.floor(0.2 / dt)) + 1
    assert nt == 504
    res = orc.step(dt, nt)
    return dict(dt=dt, nt=nt, state=orc.get_state(), res=res, u=u, v=v, wt=wt)


@pytest.fixture(scope="module")
def cavity_oracle():
    KS = kitgpu.solver_set(C2)
    orc, u, v, wt = _oracle_cavity(KS)
    dt = orc.timestep(KS.set.cfl, 0.0, KS.set.maxTime)
    res = orc.step(dt, C2_STEPS)
    return dict(dt=dt, nt=C2_STEPS, state=orc.get_state(), res=res, u=u, v=v, wt=wt)


def _gpu_run(cfg, prec, dt_ref, nt):
    KS, ctr, *faces, t = kitgpu.initialize(cfg, precision=prec)
    dt = kitgpu.timestep(KS, ctr, 0.0)
    assert dt == pytest.approx(dt_ref, rel=1e-14)
    res = kitgpu.step(KS, ctr, dt, nt)
    return ctr.handle.download(), res


def _check64(g, o, res_g, res_o):
    w, p, h, b = o
    e = rho_u_t_error(g["prim"], p)
    assert max(e) < TOL64, e
    assert np.max(np.abs(g["h"] - h)) / np.max(np.abs(h)) < TOL64
    assert np.max(np.abs(g["b"] - b)) / np.max(np.abs(b)) < TOL64
    assert np.allclose(res_g, res_o, rtol=1e-8, atol=1e-300)


def test_sod_full_fp64(gpu_lib, sod_oracle):
    g, r = _gpu_run(C1, "fp64", sod_oracle["dt"], sod_oracle["nt"])
    _check64(g, sod_oracle["state"], r, sod_oracle["res"])


def test_sod_full_fp32_split(gpu_lib, sod_oracle):
    g, r = _gpu_run(C1, "fp32", sod_oracle["dt"], sod_oracle["nt"])
    o = sod_oracle["state"]
    e = rho_u_t_error(g["prim"], o[1])
    eq = q_error(g, o, sod_oracle["u"], None, sod_oracle["wt"])
    assert max(e) < TOL32 and eq < TOLQ32, (e, eq)


def test_cavity_full_fp64(gpu_lib, cavity_oracle):
    g, r = _gpu_run(C2, "fp64", cavity_oracle["dt"], C2_STEPS)
    _check64(g, cavity_oracle["state"], r, cavity_oracle["res"])


def test_cavity_full_fp32_split(gpu_lib, cavity_oracle):
    g, r = _gpu_run(C2, "fp32", cavity_oracle["dt"], C2_STEPS)
    o = cavity_oracle["state"]
    e = rho_u_t_error(g["prim"], o[1])
    eq = q_error(g, o, cavity_oracle["u"], cavity_oracle["v"], cavity_oracle["wt"])
    assert max(e) < TOL32 and eq < TOLQ32, (e, eq)


@pytest.mark.parametrize("mom_ts", [2, 8], ids=["pass-a-lines", "pass-a-ring"])
def test_quadrant_128_fp32_split(gpu_lib, mom_ts):
    """Four-quadrant physics of the headline workload at 128^2 cells, FP32
    split with the launch shapes of the headline (4-column strips, two
    velocities per thread, 64 rows; pass A along lines with 2 faces per warp,
    or over row rings) against the oracle."""
    KS, ctr, *faces, t = kitgpu.initialize(C3S, precision="fp32")
    ctr.handle.set_tuning(4, 64, 64, mom_ts)
    P = OP.problem(KS.config, KS.ib_kw)  # the oracle's own set-up of the same config
    u, v, wt = P["u"], P["v"], P["weights"]
    orc = O.Oracle(P["cfg"], u, v, wt)
    orc.set_state(P["w"], P["prim"], P["h"], P["b"])
    dt = kitgpu.timestep(KS, ctr, 0.0)
    assert dt == pytest.approx(orc.timestep(0.5, 0.0, 1.0), rel=1e-14)
    kitgpu.step(KS, ctr, dt, C3S_STEPS)
    orc.step(dt, C3S_STEPS)
    g = ctr.handle.download()
    o = orc.get_state()
    e = rho_u_t_error(g["prim"], o[1])
    eq = q_error(g, o, u, v, wt)
    assert max(e) < TOL32 and eq < TOLQ32, (e, eq)
