"""Independent set-up of a DVM solve for the oracle (test infrastructure).

From the same key/value configuration that the product reads, this module
builds everything a solve starts from -- velocity grid and weights, gas
constants, cell centres, the initial cells (w, prim, h, b) and the Maxwell
wall states -- by the reference's own formulas, without importing the
product's set-up code.  The parity tests hand these inputs to the oracle and
the product's own to the GPU, so a set-up error in the product (a wrong
weight, viscosity, preset or wall state) makes them disagree instead of being
shared by both sides.  Only the tests and the CPU baselines use it; the
product never does.

Restated from:
  SolverSet / VSpace1D, VSpace2D   src/Solver/solver_set.jl:73-117,
                                   src/Phase/phase_velocity.jl:14-258
  newton_cotes                     src/Phase/phase_quadrature.jl:276-288
  PSpace1D / PSpace2D centres      src/Geometry/geo_struct.jl:10-186
  gas_property                     src/Struct/struct_property.jl:458-514
  heat_capacity_ratio, ref_vhs_vis src/Theory/theory_macro.jl:376-384, :447-449
  init_fvm                         src/Solver/solver_init.jl:119-141, :285-325
  ib_sod                           src/Config/cfg_sod.jl:6-62
  ib_rh (upstream lambda may be    src/Config/cfg_rh.jl:6-73
    set other than 1)
  ib_cavity, lid where y == y1     src/Config/cfg_cavity.jl:6-62
The four-quadrant state has no reference preset; it is restated from its
definition: per quadrant (x>mid,y>mid), (x<=mid,y>mid), (x<=mid,y<=mid),
(x>mid,y<=mid) the draws rho, U, V, lambda ~ U(0.1,1.5), U(-0.5,0.5),
U(-0.5,0.5), U(0.4,1.2) from numpy's default_rng(seed), in that order.
"""
import math

import numpy as np

import oracle as O


def gamma_of(K, dim):
    """heat_capacity_ratio (src/Theory/theory_macro.jl:376-384)."""
    return (K + 3.0) / (K + 1.0) if dim == 1 else (K + 4.0) / (K + 2.0)


def mu_ref_of(Kn, alpha, omega):
    """ref_vhs_vis (src/Theory/theory_macro.jl:447-449)."""
    return (5.0 * (alpha + 1.0) * (alpha + 2.0) * math.sqrt(math.pi)) / (
        4.0 * alpha * (5.0 - 2.0 * omega) * (7.0 - 2.0 * omega)) * Kn


def rh_prims(Ma, gam, lamL=1.0):
    """Upstream / downstream states of ib_rh (src/Config/cfg_rh.jl:13-27); the
    reference's upstream lambda is 1, lamL other than 1 scales U by
    sqrt(1 / lamL) and the downstream lambda with it."""
    MaR = math.sqrt((Ma ** 2 * (gam - 1.0) + 2.0) / (2.0 * gam * Ma ** 2 - (gam - 1.0)))
    ratioT = ((1.0 + (gam - 1.0) / 2.0 * Ma ** 2) * (2.0 * gam / (gam - 1.0) * Ma ** 2 - 1.0)
              / (Ma ** 2 * (2.0 * gam / (gam - 1.0) + (gam - 1.0) / 2.0)))
    s = gam / 2.0 if lamL == 1.0 else gam / (2.0 * lamL)
    primL = np.array([1.0, Ma * math.sqrt(s), lamL])
    primR = np.array([primL[0] * (gam + 1.0) * Ma ** 2 / ((gam - 1.0) * Ma ** 2 + 2.0),
                      MaR * math.sqrt(s) * math.sqrt(ratioT), primL[2] / ratioT])
    return primL, primR


def quadrant_prims(seed=20261203):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(4):
        out.append(np.array([rng.uniform(0.1, 1.5), rng.uniform(-0.5, 0.5),
                             rng.uniform(-0.5, 0.5), rng.uniform(0.4, 1.2)]))
    return out


def problem(D, ib_kw=None):
    """Everything the oracle needs for configuration dict D: a kb_config (the
    oracle's ctypes struct), flat velocity tables, initial w, prim, h, b of
    all cells (ghosts included, x fastest) and the wall states per side."""
    ib_kw = dict(ib_kw or {})
    space = D["space"]
    dim, nf = int(space[0]), int(space[2])
    K = float(D["inK"])
    gam = gamma_of(K, dim)
    mu = mu_ref_of(D["knudsen"], D.get("alphaRef", 1.0), D.get("omegaRef", 0.5))
    mesh = "newton" if D.get("vMeshType", "rectangle") == "newton" else "rectangle"
    bc = D.get("boundary", ["fix"] * (2 * dim))
    bc = [bc] * (2 * dim) if isinstance(bc, str) else list(bc)
    x0, x1, nx, ngx = D["x0"], D["x1"], D["nx"], D.get("nxg", 0)
    if dim == 1:
        u, wt = O.vspace1d(D["umin"], D["umax"], D["nu"], mesh)
        v = None
        ny, ngy, y0, y1 = 1, 0, 0.0, 1.0
        vmax = 0.0
    else:
        u, v, wt = O.vspace2d(D["umin"], D["umax"], D["nu"], D["vmin"], D["vmax"], D["nv"], mesh)
        ny, ngy, y0, y1 = D["ny"], D.get("nyg", 0), D["y0"], D["y1"]
        vmax = D["vmax"]
    cfg = O.make_config(dim, nx, ny, ngx, ngy, D["nu"], D["nv"] if dim == 2 else 1, D["flux"],
                        D["collision"], bc + ["fix"] * (4 - len(bc)), D.get("interpOrder", 2),
                        x0, x1, y0, y1, D["umax"], vmax, K, gam, mu, D.get("omega", 0.5),
                        D.get("prandtl", 1.0), nf=nf)
    dx, dy = (x1 - x0) / nx, (y1 - y0) / ny
    xs = [x0 + (i - 0.5) * dx for i in range(1 - ngx, nx + ngx + 1)]
    ys = [y0 + (j - 0.5) * dy for j in range(1 - ngy, ny + ngy + 1)] if dim == 2 else [0.0]
    case = D.get("case")
    xm, ym = (x0 + x1) / 2, (y0 + y1) / 2

    def eq(prim):
        h = O.maxwellian1(u, prim) if dim == 1 else O.maxwellian2(u, v, prim)
        return h, (np.zeros_like(h) if nf == 1 else h * K / 2.0 / prim[-1])

    if case == "sod":
        pL, pR = np.array([1.0, 0.0, 0.5]), np.array([0.125, 0.0, 0.625])
        wsel = lambda x, y: O.prim_conserve(pL if x <= xm else pR, gam)
        bcf = lambda x, y: pL if x <= xm else pR
    elif case in ("shock", "rh"):
        pL, pR = rh_prims(D.get("mach", 0.0), gam, ib_kw.get("lamL", 1.0))
        wsel = lambda x, y: O.prim_conserve(pL if x <= xm else pR, gam)
        bcf = lambda x, y: pL if x <= xm else pR
    elif case == "cavity":
        p0 = np.array([1.0, 0.0, 0.0, 1.0])
        lid = np.array([1.0, D.get("uLid", 0.15), D.get("vLid", 0.0), D.get("tLid", 1.0)])
        wsel = lambda x, y: O.prim_conserve(p0, gam)
        bcf = lambda x, y: lid if y == y1 else p0
    elif case == "quadrant":
        qp = quadrant_prims(ib_kw.get("seed", 20261203))

        def quad(x, y):
            if x > xm and y > ym:
                return 0
            if x <= xm and y > ym:
                return 1
            return 2 if y <= ym and x <= xm else 3

        wsel = lambda x, y: O.prim_conserve(qp[quad(x, y)], gam)
        bcf = lambda x, y: qp[quad(x, y)]
    else:
        raise ValueError("no independent restatement of case %r" % case)

    W, P, H, B = [], [], [], []
    for y in ys:
        for x in xs:
            w = wsel(x, y)
            p = O.conserve_prim(w, gam)
            h, b = eq(p)
            W.append(w); P.append(p); H.append(h); B.append(b)
    walls = [None] * 4
    if dim == 1:
        walls[0], walls[1] = bcf(x0, 0.0)[None, :], bcf(x1, 0.0)[None, :]
    else:
        cx = [x0 + (i - 0.5) * dx for i in range(1, nx + 1)]
        cy = [y0 + (j - 0.5) * dy for j in range(1, ny + 1)]
        # face midpoints as evolve_boundary! forms them (src/Solver/evolve_boundary.jl:52-178)
        walls[0] = np.array([bcf(cx[0] - 0.5 * dx, ((y - 0.5 * dy) + (y + 0.5 * dy)) / 2) for y in cy])
        walls[1] = np.array([bcf(cx[-1] + 0.5 * dx, ((y - 0.5 * dy) + (y + 0.5 * dy)) / 2) for y in cy])
        walls[2] = np.array([bcf(((x - 0.5 * dx) + (x + 0.5 * dx)) / 2, cy[0] - 0.5 * dy) for x in cx])
        walls[3] = np.array([bcf(((x + 0.5 * dx) + (x - 0.5 * dx)) / 2, cy[-1] + 0.5 * dy) for x in cx])
    return dict(cfg=cfg, u=u, v=v, weights=wt, w=np.array(W), prim=np.array(P), h=np.array(H),
                b=np.array(B), walls=walls, boundary=bc, gamma=gam, mu_ref=mu)
