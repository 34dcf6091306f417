"""GPU parity: libkitgpu (through the C ABI) against the FP64 CPU oracle.

Plain FP64 form: rho, U, T within 1e-12 relative (U measured against the
thermal speed) and distributions within 1e-12 of their maximum, after several
full steps, for every flux (KFVS, KCU, UGKS), collision (BGK, Shakhov) and
boundary (fix, extra, period, Maxwell) the path covers, in 1D2F1V and 2D2F2V.
"""
import numpy as np
import pytest

import kitgpu
from kitgpu import _native as N
from cases import cavity, oracle_for, quadrant, rel, rho_u_t_error, shock, sod

pytestmark = pytest.mark.gpu

TOL = 1e-12

CASES_1D = [
    ("sod-kfvs-shakhov-fix", sod(flux="kfvs", coll="shakhov")),
    ("sod-kfvs-bgk-fix-ng2", sod(flux="kfvs", coll="bgk", ng=2)),
    ("sod-kcu-shakhov-fix", sod(flux="kcu", coll="shakhov")),
    ("sod-ugks-shakhov-fix", sod(flux="ugks", coll="shakhov", Kn=1e-3)),
    ("sod-kfvs-maxwell", sod(flux="kfvs", coll="bgk", bc="maxwell")),
    ("sod-kcu-maxwell-ng1", sod(flux="kcu", coll="shakhov", bc="maxwell", ng=1)),
    ("sod-kcu-extra-ng1", sod(flux="kcu", coll="bgk", bc="extra", ng=1)),
    ("sod-ugks-extra-ng2", sod(flux="ugks", coll="shakhov", bc="extra", ng=2, Kn=1e-2)),
    ("sod-kfvs-period-ng1", sod(flux="kfvs", coll="shakhov", bc="period", ng=1)),
    ("sod-oddnu-rect", sod(nu=31, vmesh="rectangle", flux="kcu")),
    ("sod-first-order", sod(interp=1, flux="kfvs")),
    ("shock-kfvs", shock(flux="kfvs")),
    ("shock-ugks", shock(flux="ugks", Kn=1.0)),
]

CASES_2D = [
    ("cavity-kcu-shakhov-maxwell", cavity()),
    ("cavity-kfvs-bgk-maxwell-ng1", cavity(flux="kfvs", coll="bgk", ng=1, vmesh="rectangle")),
    ("cavity-ugks-shakhov-maxwell", cavity(flux="ugks", Kn=0.01)),
    ("quadrant-ugks-bgk-extra", quadrant()),
    ("quadrant-kcu-shakhov-extra", quadrant(flux="kcu", coll="shakhov", Kn=1e-2)),
    ("quadrant-kfvs-shakhov-fix", quadrant(flux="kfvs", coll="shakhov", bc="fix", ng=0)),
    ("quadrant-ugks-shakhov-fix-rect", quadrant(nx=9, ny=7, nu=11, nv=13, coll="shakhov", bc="fix", ng=0)),
    # grids wide enough for the interior (branch-free) strips and segments
    ("quadrant-ugks-shakhov-extra-16", quadrant(nx=17, ny=18, nu=8, nv=8, coll="shakhov", Kn=1e-2)),
    ("cavity-kfvs-shakhov-maxwell-16", cavity(nx=16, ny=19, nu=8, nv=6, flux="kfvs")),
    ("cavity-kcu-bgk-maxwell-16", cavity(nx=18, ny=16, nu=10, nv=8, coll="bgk")),
]


def _run_both(cfg, nsteps, precision="fp64"):
    KS, ctr, *faces, t = kitgpu.initialize(cfg, precision=precision)
    orc = oracle_for(KS)
    dt = kitgpu.timestep(KS, ctr, 0.0)
    assert dt == pytest.approx(orc.timestep(KS.set.cfl, 0.0, KS.set.maxTime), rel=1e-14)
    res_g = kitgpu.step(KS, ctr, dt, nsteps)
    res_o = orc.step(dt, nsteps)
    return KS, ctr, orc, dt, res_g, res_o


def _compare_state(ctr, orc, tol):
    g = ctr.handle.download()
    w, p, h, b = orc.get_state()
    e_rho, e_u, e_t = rho_u_t_error(g["prim"], p)
    assert e_rho < tol and e_u < tol and e_t < tol, (e_rho, e_u, e_t)
    assert rel(g["w"][:, 0], w[:, 0]) < tol
    hs = np.max(np.abs(h))
    assert np.max(np.abs(g["h"] - h)) / hs < tol
    assert np.max(np.abs(g["b"] - b)) / np.max(np.abs(b)).clip(1e-300) < tol


@pytest.mark.parametrize("name,cfg", CASES_1D, ids=[c[0] for c in CASES_1D])
def test_fp64_parity_1d(gpu_lib, name, cfg):
    KS, ctr, orc, dt, rg, ro = _run_both(cfg, 25)
    _compare_state(ctr, orc, TOL)
    assert np.allclose(rg, ro, rtol=1e-9, atol=1e-300)


@pytest.mark.parametrize("name,cfg", CASES_2D, ids=[c[0] for c in CASES_2D])
def test_fp64_parity_2d(gpu_lib, name, cfg):
    KS, ctr, orc, dt, rg, ro = _run_both(cfg, 8)
    _compare_state(ctr, orc, TOL)
    assert np.allclose(rg, ro, rtol=1e-9, atol=1e-300)


@pytest.mark.parametrize("name,cfg", CASES_1D[:9] + CASES_2D, ids=[c[0] for c in CASES_1D[:9] + CASES_2D])
def test_stage_parity(gpu_lib, name, cfg):
    """reconstruct! / evolve! outputs (slopes, face fw / fh / fb) after two steps."""
    KS, ctr, orc, dt, _, _ = _run_both(cfg, 2)
    faces = ()
    kitgpu.reconstruct(KS, ctr)
    orc.reconstruct()
    sw_g, sh_g, sb_g = ctr.handle.slopes()
    sw_o, sh_o, sb_o = orc.slopes()
    scale = max(np.max(np.abs(sh_o)), 1e-300)
    assert np.max(np.abs(sh_g - sh_o)) / scale < 1e-11
    assert np.max(np.abs(sb_g - sb_o)) / max(np.max(np.abs(sb_o)), 1e-300) < 1e-11
    if KS.set.flux != "kfvs":
        assert np.max(np.abs(sw_g - sw_o)) / max(np.max(np.abs(sw_o)), 1e-300) < 1e-11
    kitgpu.evolve(KS, ctr, *faces, dt)
    orc.evolve(dt)
    fw_g, fh_g, fb_g = ctr.handle.faces(dt)
    fw_o, fh_o, fb_o = orc.faces()
    for k in range(fw_o.shape[1]):
        s = max(np.max(np.abs(fw_o[:, k])), 1e-300)
        assert np.max(np.abs(fw_g[:, k] - fw_o[:, k])) / s < 1e-11, k
    assert np.max(np.abs(fh_g - fh_o)) / max(np.max(np.abs(fh_o)), 1e-300) < 1e-11
    assert np.max(np.abs(fb_g - fb_o)) / max(np.max(np.abs(fb_o)), 1e-300) < 1e-11
    r_g = np.zeros(KS.dim + 2)
    kitgpu.update(KS, ctr, *faces, dt, r_g)
    r_o = orc.update(dt)
    assert np.allclose(r_g, r_o, rtol=1e-9, atol=1e-300)
    _compare_state(ctr, orc, TOL)


FP32_CASES = [
    ("sod-kfvs-shakhov", sod(flux="kfvs", coll="shakhov"), 100),
    ("sod-kcu-bgk-maxwell", sod(flux="kcu", coll="bgk", bc="maxwell"), 100),
    ("sod-ugks-shakhov-extra", sod(flux="ugks", coll="shakhov", bc="extra", ng=1, Kn=1e-2), 100),
    ("cavity-kcu-shakhov", cavity(nx=12, ny=12, nu=16, nv=16), 50),
    ("quadrant-ugks-bgk-extra", quadrant(nx=12, ny=12, nu=16, nv=16), 50),
]


@pytest.mark.parametrize("name,cfg,n", FP32_CASES, ids=[c[0] for c in FP32_CASES])
def test_fp32_split_error(gpu_lib, name, cfg, n):
    """FP32 h / b with FP64 moments: L-inf error <= 1e-5 in rho, U, T."""
    KS, ctr, orc, dt, rg, ro = _run_both(cfg, n, precision="fp32")
    g = ctr.handle.download()
    w, p, h, b = orc.get_state()
    e = rho_u_t_error(g["prim"], p)
    assert max(e) < 1e-5, e


FP32_SHAPES = [(tx, bs) for tx in (2, 4) for bs in (64, 128)]


@pytest.mark.parametrize("tx,bs", FP32_SHAPES, ids=["tx%d-bs%d" % s for s in FP32_SHAPES])
@pytest.mark.parametrize("name,cfg", [
    ("cavity-kcu-shakhov", cavity(nx=13, ny=11, nu=14, nv=16)),
    ("quadrant-ugks-bgk-extra", quadrant(nx=18, ny=17, nu=15, nv=12)),
    ("quadrant-kfvs-shakhov-extra", quadrant(nx=17, ny=19, nu=16, nv=13, flux="kfvs", coll="shakhov")),
], ids=lambda x: x if isinstance(x, str) else "")
def test_fp32_update_shapes(gpu_lib, name, cfg, tx, bs):
    """Every launch shape of the FP32 2D update (one or two velocities per
    thread, two or four columns per strip), incl. partial strips and velocity
    pairs whose upwind sides differ, stays within 1e-5 of the FP64 oracle."""
    KS, ctr, *faces, t = kitgpu.initialize(cfg, precision="fp32")
    ctr.handle.set_tuning(march_tx=tx, march_ry=8, march_bs=bs)
    orc = oracle_for(KS)
    dt = kitgpu.timestep(KS, ctr, 0.0)
    kitgpu.step(KS, ctr, dt, 30)
    orc.step(dt, 30)
    g = ctr.handle.download()
    w, p, h, b = orc.get_state()
    e = rho_u_t_error(g["prim"], p)
    assert max(e) < 1e-5, e


@pytest.mark.parametrize("name,cfg,prec", [
    ("sod", sod(), "fp64"), ("cavity", cavity(nx=9, ny=7), "fp64"),
    ("quadrant-ghosts", quadrant(nx=6, ny=5), "fp64"), ("cavity-fp32", cavity(nx=9, ny=7), "fp32"),
], ids=lambda x: x if isinstance(x, str) else "")
def test_init_equilibrium_matches_host_state(gpu_lib, name, cfg, prec):
    """kb_init_equilibrium builds on the device the h, b that init_fvm builds
    on the host (equal to 1e-14 in FP64, to FP32 rounding in FP32)."""
    KS, ctr, *faces, t = kitgpu.initialize(cfg, precision=prec)
    ref = ctr.handle.download()
    w, p = kitgpu.solver.initial_cells(KS)
    ctr.handle.init_equilibrium(w, p)
    got = ctr.handle.download()
    tol = 1e-14 if prec == "fp64" else 0.0
    for k in ("w", "prim", "h", "b"):
        scale = np.max(np.abs(ref[k]))
        assert np.max(np.abs(got[k] - ref[k])) <= tol * scale + (6e-8 * np.abs(ref[k]).max() if prec == "fp32" else 0.0), k


MOM_CASES = [
    ("quadrant-ugks-bgk-extra", quadrant(nx=18, ny=17, nu=15, nv=12)),
    ("quadrant-kcu-bgk-extra", quadrant(nx=13, ny=22, nu=12, nv=16, flux="kcu")),
    ("cavity-kfvs-bgk-walls", cavity(nx=13, ny=11, nu=14, nv=16, flux="kfvs", coll="bgk")),
    ("cavity-ugks-bgk-walls", cavity(nx=21, ny=19, nu=16, nv=14, flux="ugks", coll="bgk")),
]


def _fw_after_evolve(cfg, mom_ts):
    KS, ctr, *faces, t = kitgpu.initialize(cfg, precision="fp32")
    h = ctr.handle
    h.set_tuning(march_ry=8, mom_ts=mom_ts)
    dt = kitgpu.timestep(KS, ctr, 0.0)
    kitgpu.step(KS, ctr, dt, 3)  # a state with gradients everywhere
    h.reconstruct()
    h.evolve(dt)
    fw = np.zeros((h.nface, h.nw))
    h.call("kb_download_faces", float(dt), N.ptr(fw), None, None)
    return KS, ctr, dt, fw


@pytest.mark.parametrize("name,cfg", MOM_CASES, ids=[c[0] for c in MOM_CASES])
def test_fp32_moment_pass_forms_agree(gpu_lib, name, cfg):
    """The one-launch row-ring form of pass A (mom_ts 8: both face directions
    from one read of h, b, partial sums per velocity box) gives the face
    moments fw of the two-launch form (x lines, then y lines) to FP32
    summation order: within 2e-6 of each moment's largest magnitude, on
    partial strips, odd velocity counts and Maxwell walls."""
    _, _, _, fa = _fw_after_evolve(cfg, 4)
    _, _, _, fb = _fw_after_evolve(cfg, 8)
    scale = np.max(np.abs(fa), axis=0)
    assert np.all(np.max(np.abs(fb - fa), axis=0) <= 2e-6 * scale), (np.max(np.abs(fb - fa), axis=0), scale)


@pytest.mark.parametrize("name,cfg", MOM_CASES, ids=[c[0] for c in MOM_CASES])
def test_fp32_ring_moment_pass_against_oracle(gpu_lib, name, cfg):
    """30 FP32 steps with the row-ring pass A stay within 1e-5 of the FP64
    oracle in rho, U, T."""
    KS, ctr, *faces, t = kitgpu.initialize(cfg, precision="fp32")
    ctr.handle.set_tuning(march_ry=8, mom_ts=8)
    orc = oracle_for(KS)
    dt = kitgpu.timestep(KS, ctr, 0.0)
    kitgpu.step(KS, ctr, dt, 30)
    orc.step(dt, 30)
    e = rho_u_t_error(ctr.handle.download()["prim"], orc.get_state()[1])
    assert max(e) < 1e-5, e


@pytest.mark.parametrize("name,cfg", [("sod-kfvs-shakhov", sod(nx=60, flux="kfvs", coll="shakhov")),
                                      ("quadrant-ugks-bgk", quadrant(nx=12, ny=11, nu=12, nv=10))],
                         ids=lambda x: x if isinstance(x, str) else "")
def test_per_step_dt_option(gpu_lib, name, cfg):
    """kb_step_cfl (solve(..., adaptive=True)): dt recomputed from the current
    state on the device before every step; the oracle doing the same loop
    (timestep, then one step) matches to 1e-12 in rho, U, T and in the time
    reached; the run stops at maxTime."""
    KS, ctr, *faces, t = kitgpu.initialize(cfg, precision="fp64")
    orc = oracle_for(KS)
    n = 15
    tg, rg = ctr.handle.step_cfl(KS.set.cfl, 0.0, KS.set.maxTime, n)
    to = 0.0
    for _ in range(n):
        dt = orc.timestep(KS.set.cfl, to, KS.set.maxTime)
        orc.step(dt, 1)
        to += dt
    assert tg == pytest.approx(to, rel=1e-13)
    e = rho_u_t_error(ctr.handle.download()["prim"], orc.get_state()[1])
    assert max(e) < 1e-12, e
    # a short maxTime ends the loop there
    KS2, ctr2, *faces2, t2 = kitgpu.initialize(dict(cfg, maxTime=3.5 * tg / n), precision="fp64")
    t_end = kitgpu.solve(KS2, ctr2, adaptive=True, chunk=4)
    assert t_end == pytest.approx(KS2.set.maxTime, rel=1e-12)
