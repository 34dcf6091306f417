"""Unstructured 2D2F2V (triangle meshes) through the C ABI against the
oracle's own restatement of the reference's US2F step (oracle/oracle_us.py:
its own connectivity and geometry from the same points and triangles).

The setup follows the reference's unstructured test (test/t1_2f.txt: KFVS,
first order, 16 x 16 velocities on [-5, 5]^2, Kn 0.075, Pr 1, inK 1) on
jittered triangulations of a rectangle, started from a density / pressure
bump so that every face carries flux.  Plain FP64 form: rho, U, T and h, b
within 1e-12 of the oracle; FP32 split form: rho, U, T within 1e-5.
The 2D1F2V cases (the reference's test/t1_1f.txt: the same setup with
space = 2d1f2v, BGK) check the device's "2F with b held at zero" form against
the oracle's own 1F restatement; b must stay exactly zero.
"""
import numpy as np
import pytest

from kitgpu import unstruct as US
import oracle_us as OU
from cases import rel, rho_u_t_error

pytestmark = pytest.mark.gpu


def bump(x, y):
    r2 = (x - 0.45) ** 2 + (y - 0.55) ** 2
    return np.array([1.0 + 0.5 * np.exp(-r2 / 0.02), 0.1, -0.05, 1.0 / (1.0 + 0.3 * np.exp(-r2 / 0.02))])


CASES = [
    ("fix-bgk", dict(boundary="fix", collision="bgk", nx=10, ny=8, jitter=0.25)),
    ("extra-bgk", dict(boundary="extra", collision="bgk", nx=9, ny=9, jitter=0.2)),
    ("fix-shakhov", dict(boundary="fix", collision="shakhov", nx=8, ny=10, jitter=0.3)),
    ("extra-shakhov-newton", dict(boundary="extra", collision="shakhov", nx=12, ny=7, jitter=0.15,
                                  vmesh="newton", nu=12)),
    ("1f-fix-bgk-t1_1f", dict(boundary="fix", collision="bgk", nx=9, ny=11, jitter=0.25,
                              space="2d1f2v")),
    ("1f-extra-bgk-inK0", dict(boundary="extra", collision="bgk", nx=10, ny=9, jitter=0.2,
                               space="2d1f2v", inK=0.0)),
    # 18 x 18 velocities: past the staged FP32 form's 256, the direct-load form
    ("fix-shakhov-v18", dict(boundary="fix", collision="shakhov", nx=8, ny=7, jitter=0.2, nu=18)),
]


def _setup(c, tmp_path=None):
    P, T = US.rectangle_mesh(c["nx"], c["ny"], jitter=c["jitter"])
    if tmp_path is not None:  # through a gmsh file, as a user's mesh would come
        path = str(tmp_path / "mesh.msh")
        US.write_gmsh(path, P, T)
        P, T = US.read_gmsh(path)
    m = US.build_mesh(P, T, boundary=c["boundary"])
    nu = c.get("nu", 16)
    KS = US.unstruct_solver_set(m, nu=nu, nv=nu, vmesh=c.get("vmesh", "rectangle"),
                                collision=c["collision"], prim_at=bump,
                                space=c.get("space", "2d2f2v"), inK=c.get("inK", 1.0))
    vs, g = KS.vs, KS.gas
    orc = OU.UnstructOracle(P, T, m.cell_type, vs.flat(vs.u), vs.flat(vs.v), vs.flat(vs.weights),
                            g.K, g.gamma, g.mu_ref, g.omega, g.Pr, c["collision"], nf=KS.nf)
    orc.set_state(*US.initial_cells(KS))
    return KS, orc


@pytest.mark.parametrize("name,c", CASES, ids=[x[0] for x in CASES])
def test_unstructured_fp64_parity(gpu_lib, tmp_path, name, c):
    KS, orc = _setup(c, tmp_path)
    hd = US.init_fvm(KS, "fp64")
    dt = hd.timestep()
    assert dt == pytest.approx(orc.timestep(KS.set.cfl, 0.0, KS.set.maxTime, KS.vs.u1, KS.vs.v1),
                               rel=1e-14)
    rg = hd.step(dt, 12)
    ro = orc.step(dt, 12)
    g = hd.download()
    w, p, h, b = orc.get_state()
    e = rho_u_t_error(g["prim"], p)
    assert max(e) < 1e-12, e
    assert rel(g["w"][:, 0], w[:, 0]) < 1e-12
    assert np.max(np.abs(g["h"] - h)) / np.max(np.abs(h)) < 1e-12
    if KS.nf == 2:
        assert np.max(np.abs(g["b"] - b)) / np.max(np.abs(b)) < 1e-12
    else:
        assert np.all(g["b"] == 0.0)
    assert np.allclose(rg, ro, rtol=1e-9, atol=1e-300)
    assert hd.launches() > 0


@pytest.mark.parametrize("name,c", CASES, ids=[x[0] for x in CASES])
def test_unstructured_fp32_split(gpu_lib, name, c):
    KS, orc = _setup(c)
    hd = US.init_fvm(KS, "fp32")
    dt = hd.timestep()
    hd.step(dt, 40)
    orc.step(dt, 40)
    g = hd.download()
    e = rho_u_t_error(g["prim"], orc.get_state()[1])
    assert max(e) < 1e-5, e
    assert KS.nf == 2 or np.all(g["b"] == 0.0)


def test_unstructured_conservation(gpu_lib):
    """Interior faces add to one cell exactly what they take from the other,
    so over one step the stepped cells' mass, momentum and energy change only
    by the fluxes through their faces to the fixed cells (taken from the
    oracle's own face fluxes of that step)."""
    c = dict(boundary="fix", collision="shakhov", nx=14, ny=14, jitter=0.2)
    KS, orc = _setup(c)
    hd = US.init_fvm(KS, "fp64")
    dt = hd.timestep()
    ps = KS.ps
    area = ps.cell_area
    inner = ps.cell_type == 0
    w0 = hd.download()["w"]
    hd.step(dt, 1)
    w1 = hd.download()["w"]
    orc.evolve(dt)
    leak = np.zeros(4)
    for cc in np.nonzero(inner)[0]:
        for j in range(3):
            if not inner[ps.cell_neighbors[cc, j]]:
                leak += orc.dirc[cc, j] * orc.fw[orc.cell_face[cc][j]]
    change = np.sum((w1 - w0)[inner] * area[inner, None], axis=0)
    scale = np.sum(np.abs(w0[inner]) * area[inner, None], axis=0)
    assert np.all(np.abs(change + leak) <= 1e-13 * scale), (change, leak)
    assert np.all(np.abs(leak) > 1e-10 * scale)  # flux does cross to the fixed ring


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 1e-5)])
def test_unstructured_long_run_against_c_oracle(gpu_lib, prec, tol):
    """A 48 x 48-quad mesh (4608 triangles, extrapolated boundaries, Shakhov)
    over 200 steps against the multithreaded C oracle: rho, U, T within
    1e-12 (FP64) and 1e-5 (FP32 split)."""
    c = dict(boundary="extra", collision="shakhov", nx=48, ny=48, jitter=0.2)
    KS, orc = _setup(c)
    orc.use_c()
    hd = US.init_fvm(KS, prec)
    dt = hd.timestep()
    assert dt == pytest.approx(orc.timestep(KS.set.cfl, 0.0, KS.set.maxTime, KS.vs.u1, KS.vs.v1), rel=1e-14)
    hd.step(dt, 200)
    orc.step(dt, 200)
    e = rho_u_t_error(hd.download()["prim"], orc.get_state()[1])
    assert max(e) < tol, e


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_unstructured_shape_independent_and_tuned(gpu_lib, prec):
    """The cells-per-CTA shape changes only how cells are grouped: the state
    after 5 steps is bit-identical for 4 and 32 cells per CTA; out-of-range
    shapes are refused; the autotuner keeps one of its candidates."""
    from kitgpu import _native as N
    from kitgpu import tune
    c = dict(boundary="extra", collision="shakhov", nx=11, ny=9, jitter=0.2)
    KS, orc = _setup(c)
    out = []
    for cb in (4, 32):
        hd = US.init_fvm(KS, prec)
        hd.set_tuning(cb)
        assert hd.tuning() == cb
        dt = hd.timestep()
        hd.step(dt, 5)
        out.append(hd.download())
        hd.close()
    for k in ("w", "prim", "h", "b"):
        assert np.array_equal(out[0][k], out[1][k]), k
    hd = US.init_fvm(KS, prec)
    for bad in (-1, 33):
        with pytest.raises(N.KitGPUError):
            hd.set_tuning(bad)
    dt = hd.timestep()
    best, times = tune.autotune_unstruct(hd, dt, steps=2, use_cache=False)
    assert best in tune.US_CELLS_PER_CTA and hd.tuning() == best and len(times) >= 1


@pytest.mark.parametrize("space", ["2d2f2v", "2d1f2v"])
def test_initialize_from_config(gpu_lib, tmp_path, space):
    """kitgpu.initialize on a config in the reference's format with
    `mesh = <gmsh file>` (as test/test_unstructure.jl reads t1_2f.txt /
    t1_1f.txt, here with extrapolated boundary cells) gives the device cells
    of the unstructured solve; 10 steps match the oracle to 1e-12."""
    import kitgpu
    from test_unstruct_mesh import T1_CFG
    P, T = US.rectangle_mesh(9, 7, jitter=0.2)
    US.write_gmsh(str(tmp_path / "m.msh"), P, T)
    cfg = tmp_path / "u.txt"
    cfg.write_text(T1_CFG.format(space=space, bc="extra", mesh="m.msh"))
    KS, hd, t = kitgpu.initialize(str(cfg))
    assert t == 0.0 and KS.nf == (2 if space == "2d2f2v" else 1)
    vs, g = KS.vs, KS.gas
    orc = OU.UnstructOracle(P, T, KS.ps.cell_type, vs.flat(vs.u), vs.flat(vs.v), vs.flat(vs.weights),
                            g.K, g.gamma, g.mu_ref, g.omega, g.Pr, "bgk", nf=KS.nf)
    orc.set_state(*US.initial_cells(KS))
    dt = hd.timestep()
    assert dt == pytest.approx(orc.timestep(KS.set.cfl, 0.0, KS.set.maxTime, vs.u1, vs.v1), rel=1e-14)
    hd.step(dt, 10)
    orc.step(dt, 10)
    e = rho_u_t_error(hd.download()["prim"], orc.get_state()[1])
    assert max(e) < 1e-12, e
