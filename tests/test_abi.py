"""C ABI and host logic without a GPU: the library loads and exports every
symbol include/kitgpu.h declares, config validation rejects what the path does
not support (host code only, before any CUDA call), and the host mirror of the
reference setup (read_cfg, velocity / physical spaces, presets) matches the
oracle's independent restatement."""
import ctypes
import os
import re

import numpy as np
import pytest

import kitgpu
from kitgpu import _native as N
import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "kitgpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(kb_\w+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol():
    lib = N.load()
    syms = header_symbols()
    assert len(syms) >= 20
    for name in syms:
        assert hasattr(lib, name), name
    assert lib.kb_version().decode().startswith("kitgpu")


def test_signatures_cover_header():
    from kitgpu import batch
    from kitgpu import unstruct
    known = set(N.SIGNATURES) | set(batch._BATCH_SIGS) | set(batch._POOL_SIGS) | set(unstruct._US_SIGS)
    for name in header_symbols():
        if name in ("kb_version", "kb_last_error"):
            continue
        assert name in known, name


def _cfg(**kw):
    c = N.KbConfig()
    base = dict(dim=1, nx=10, ny=1, ngx=0, ngy=0, nu=8, nv=1, flux=0, collision=0,
                interp_order=2, precision=0, x0=0.0, x1=1.0, y0=0.0, y1=1.0, umax=5.0,
                vmax=0.0, K=2.0, gamma=5 / 3, mu_ref=1e-3, omega=0.81, Pr=2 / 3)
    base.update(kw)
    bc = base.pop("bc", (0, 0, 0, 0))
    for k, v in base.items():
        setattr(c, k, v)
    for k in range(4):
        c.bc[k] = bc[k]
    return c


BAD = [
    ("dim", dict(dim=3)),
    ("nx", dict(nx=2)),
    ("ghosts", dict(ngx=3)),
    ("flux", dict(flux=7)),
    ("extra-without-ghosts", dict(bc=(1, 1, 0, 0))),
    ("period-one-side", dict(ngx=1, bc=(2, 0, 0, 0))),
    ("2d-mixed", dict(dim=2, ny=5, nv=4, bc=(3, 3, 0, 3))),
    ("2d-period", dict(dim=2, ny=5, nv=4, ngx=1, ngy=1, bc=(2, 2, 2, 2))),
    ("interp", dict(interp_order=3)),
    ("precision", dict(precision=5)),
    ("gamma", dict(gamma=1.0)),
    ("nf", dict(nf=3)),
    # 1F: no UGKS step, no 1D1F1V Maxwell wall, no 2D1F2V Shakhov in the reference
    ("1f-ugks", dict(nf=1, flux=2)),
    ("1d1f-maxwell", dict(nf=1, bc=(3, 3, 0, 0))),
    ("2d1f-shakhov", dict(nf=1, dim=2, ny=5, nv=4, collision=1)),
]


@pytest.mark.parametrize("name,kw", BAD, ids=[b[0] for b in BAD])
def test_invalid_configs_rejected_before_cuda(name, kw):
    lib = N.load()
    c = _cfg(**kw)
    u = np.linspace(-1, 1, 16)
    h = N._H()
    rc = lib.kb_create(ctypes.byref(c), N.ptr(u), N.ptr(u), N.ptr(u), ctypes.byref(h))
    assert rc == -2, (rc, lib.kb_last_error())
    assert lib.kb_last_error().decode()


def test_null_arguments():
    lib = N.load()
    assert lib.kb_create(None, None, None, None, None) == -1
    assert lib.kb_step(None, 1.0, 1, None) == -1
    assert lib.kb_destroy(None) == 0


def test_read_cfg(tmp_path):
    p = tmp_path / "shock.txt"
    p.write_text("# 1D shock\ncase = shock\nspace = 1d2f1v\nflux = kfvs\ncollision = bgk\n"
                 "nSpecies = 1\ninterpOrder = 2\nlimiter = vanleer\nboundary = fix\ncfl = 0.95\n"
                 "maxTime = 0.0001\nhasForce = false\nx0 = -35.0\nx1 = 35.0\nnx = 50\nnxg = 2\n"
                 "umin = -12.0\numax = 12.0\nnu = 16\nvMeshType = rectangle\nknudsen = 1.0\n"
                 "mach = 2.0 # upstream\nprandtl = 1.0\ninK = 2.0\nomega = 0.72\n")
    D = kitgpu.read_cfg(str(p))
    assert D["boundary"] == ["fix", "fix"] and D["nx"] == 50 and isinstance(D["nx"], int)
    assert D["hasForce"] is False and D["mach"] == 2.0 and D["cfl"] == 0.95
    KS = kitgpu.solver_set(str(p))
    assert KS.gas.gamma == pytest.approx(5 / 3)
    assert KS.gas.mu_ref == pytest.approx(kitgpu.ref_vhs_vis(1.0, 1.0, 0.5))
    assert KS.ps.x.shape == (54,)
    pl, pr = KS.ib.p["primL"], KS.ib.p["primR"]
    assert pl[1] == pytest.approx(2.0 * np.sqrt(5 / 3 / 2))
    assert pr[0] > pl[0]


def test_setup_matches_oracle_restatement():
    for nu in (16, 33, 101):
        vs = kitgpu.VSpace1D.build(-5, 5, nu, type="newton")
        u, w = O.vspace1d(-5, 5, nu, "newton")
        assert np.array_equal(vs.u, u) and np.array_equal(vs.weights, w)
    vs2 = kitgpu.VSpace2D.build(-5, 5, 12, -4, 4, 10, type="newton")
    U, V, W = O.vspace2d(-5, 5, 12, -4, 4, 10, "newton")
    assert np.array_equal(vs2.flat(vs2.u), U) and np.array_equal(vs2.flat(vs2.v), V)
    assert np.array_equal(vs2.flat(vs2.weights), W)
    from cases import sod, cavity
    KS = kitgpu.solver_set(sod(nx=20, nu=17))
    w, p, h, b = kitgpu.initial_state(KS)
    W2, P2, H2, B2 = O.sod_state(20, 0, 0.0, 1.0, KS.vs.u, KS.gas.gamma, KS.gas.K)
    assert np.allclose(w, W2, rtol=1e-15) and np.allclose(h, H2, rtol=1e-14)
    for ny in (19, 27, 64):
        KS = kitgpu.solver_set(cavity(nx=ny, ny=ny))
        mine = kitgpu.wall_states(KS)
        ref = O.cavity_walls(ny, ny, 0.0, 1.0, 0.0, 1.0)
        for a, r in zip(mine, ref):
            assert np.array_equal(a, r)


def test_cavity_lid_quirk():
    """ib_cavity returns the lid state only where y == y1 exactly
    (src/Config/cfg_cavity.jl:30): for ny = 19 the top face midpoint is not
    exactly 1.0 and the lid is a stationary wall."""
    from cases import cavity
    KS = kitgpu.solver_set(cavity(nx=19, ny=19))
    top = kitgpu.wall_states(KS)[3]
    KS64 = kitgpu.solver_set(cavity(nx=64, ny=64))
    top64 = kitgpu.wall_states(KS64)[3]
    assert top64[0][1] == pytest.approx(0.15)
    dy = 1.0 / 19
    yc = ((0.0 + (19 - 0.5) * dy + 0.5 * dy) + (0.0 + (19 - 0.5) * dy + 0.5 * dy)) / 2
    assert yc != 1.0
    assert top[0][1] == 0.0


def test_unsupported_paths_raise():
    from cases import sod
    cfg = sod()
    cfg["space"] = "1d3f1v"
    with pytest.raises(ValueError):
        kitgpu.solver_set(cfg)
    cfg = sod()
    cfg["limiter"] = "minmod"
    with pytest.raises(ValueError):
        kitgpu.solver_set(cfg)


def test_tune_signature_and_options():
    from kitgpu import tune
    # the values kb_set_tuning accepts (8: the row-ring pass A)
    assert set(tune.MARCH_TX) <= {2, 4} and set(tune.MOM_TS) <= {2, 4, 8}


@pytest.mark.parametrize("cfg", [
    ("sod", dict()), ("sod-ghosts-rect", dict(ng=2, vmesh="rectangle", nu=31)),
    ("sod-1f", dict(space="1d1f1v")), ("shock", dict()), ("shock-lam05", dict(lamL=0.5)),
    ("cavity", dict()), ("cavity-19", dict(nx=19, ny=19)), ("cavity-lid", dict(lid=0.3)),
    ("quadrant", dict()), ("quadrant-seed", dict(seed=7)), ("cavity-1f", dict(space="2d1f2v")),
], ids=lambda c: c[0])
def test_product_setup_matches_independent_oracle_setup(cfg):
    """The product's set-up (kitgpu.setup: SolverSet, init_fvm, wall states)
    and the oracle's own restatement (oracle_setup.problem) give the same
    configuration, velocity tables, initial cells and walls from one config
    dict, for every preset the parity tests run."""
    import oracle_setup as OP
    from cases import cavity, quadrant, shock, sod
    name, kw = cfg
    ib_kw = {}
    if name.startswith("sod"):
        D = sod(**{k: v for k, v in kw.items() if k != "space"})
    elif name.startswith("shock"):
        D = shock()
        if "lamL" in kw:
            ib_kw["lamL"] = kw["lamL"]
    elif name.startswith("cavity"):
        D = cavity(**{k: v for k, v in kw.items() if k != "space"})
    else:
        D = quadrant()
        if "seed" in kw:
            ib_kw["seed"] = kw["seed"]
    if "space" in kw:
        D["space"] = kw["space"]
        if kw["space"] == "2d1f2v":
            D["collision"] = "bgk"
    KS = kitgpu.solver_set(D, **ib_kw)
    P = OP.problem(KS.config, KS.ib_kw)
    mine = kitgpu.kb_config(KS)
    ref = P["cfg"]
    for f in ("dim", "nx", "ny", "ngx", "ngy", "nu", "nv", "flux", "collision", "interp_order", "nf"):
        assert getattr(mine, f) == getattr(ref, f), f
    assert list(mine.bc) == list(ref.bc)
    for f in ("x0", "x1", "umax", "K", "omega", "Pr"):
        assert getattr(mine, f) == getattr(ref, f), f
    for f in ("gamma", "mu_ref"):
        assert getattr(mine, f) == pytest.approx(getattr(ref, f), rel=1e-15), f
    vs = KS.vs
    if KS.dim == 1:
        assert np.array_equal(vs.u, P["u"]) and np.array_equal(vs.weights, P["weights"])
    else:
        assert np.array_equal(vs.flat(vs.u), P["u"]) and np.array_equal(vs.flat(vs.v), P["v"])
        assert np.array_equal(vs.flat(vs.weights), P["weights"])
    w, p, h, b = kitgpu.initial_state(KS)
    for a, r in ((w, P["w"]), (p, P["prim"]), (h, P["h"]), (b, P["b"])):
        assert a.shape == r.shape
        assert np.allclose(a, r, rtol=1e-14, atol=1e-300)
    for side, prim in enumerate(kitgpu.wall_states(KS)):
        assert np.allclose(prim, P["walls"][side], rtol=1e-15, atol=0)
