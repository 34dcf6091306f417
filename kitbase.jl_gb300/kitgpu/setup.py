"""Host-side setup of a DVM solve: the parts of KitBase's SolverSet that the
reference builds on the CPU before the time loop (configuration, velocity and
physical meshes, gas properties, initial and boundary states).  Pure numpy;
the DVM step itself runs in libkitgpu.

Mirrors (file:line in KitBase.jl v0.9.31):
  read_cfg / read_dict          src/IO/io_read.jl:12-43, :95-128
  Setup                         src/Struct/struct_setup.jl:106-160
  Gas, gas_property             src/Struct/struct_property.jl:51-64, :458-514
  VSpace1D / VSpace2D           src/Phase/phase_velocity.jl:14-65, :128-258
  newton_cotes                  src/Phase/phase_quadrature.jl:276-288
  PSpace1D / PSpace2D           src/Geometry/geo_struct.jl:10-186
  prim_conserve / conserve_prim src/Theory/theory_macro.jl:10-33, :185-206
  maxwellian                    src/Theory/theory_equilibrium.jl:8-25
  ib_sod / ib_cavity / ib_rh    src/Config/cfg_sod.jl:6-62, cfg_cavity.jl:6-62, cfg_rh.jl:6-73
"""
import math
from dataclasses import dataclass, field

import numpy as np

# ------------------------------------------------------------------ theory


def heat_capacity_ratio(K, D):
    """src/Theory/theory_macro.jl:376-384"""
    return {1: (K + 3.0) / (K + 1.0), 2: (K + 4.0) / (K + 2.0), 3: (K + 5.0) / (K + 3.0)}[D]


def ref_vhs_vis(Kn, alpha, omega):
    """src/Theory/theory_macro.jl:447-449"""
    return (5.0 * (alpha + 1.0) * (alpha + 2.0) * math.sqrt(math.pi) /
            (4.0 * alpha * (5.0 - 2.0 * omega) * (7.0 - 2.0 * omega)) * Kn)


def prim_conserve(prim, gamma):
    """src/Theory/theory_macro.jl:10-33"""
    p = [float(x) for x in prim]
    if len(p) == 3:
        return np.array([p[0], p[0] * p[1],
                         0.5 * p[0] / p[2] / (gamma - 1.0) + 0.5 * p[0] * (p[1] * p[1])])
    return np.array([p[0], p[0] * p[1], p[0] * p[2],
                     0.5 * p[0] / p[3] / (gamma - 1.0) + 0.5 * p[0] * (p[1] * p[1] + p[2] * p[2])])


def conserve_prim(w, gamma):
    """src/Theory/theory_macro.jl:185-206"""
    W = [float(x) for x in w]
    if len(W) == 3:
        return np.array([W[0], W[1] / W[0],
                         0.5 * W[0] / (gamma - 1.0) / (W[2] - 0.5 * (W[1] * W[1]) / W[0])])
    return np.array([W[0], W[1] / W[0], W[2] / W[0],
                     0.5 * W[0] / (gamma - 1.0) / (W[3] - 0.5 * (W[1] * W[1] + W[2] * W[2]) / W[0])])


def maxwellian(u, prim, v=None):
    """Discrete Maxwellian, 1V or 2V (src/Theory/theory_equilibrium.jl:8-25)."""
    if v is None:
        return prim[0] * np.sqrt(prim[-1] / np.pi) * np.exp(-prim[-1] * (u - prim[1]) ** 2)
    return prim[0] * (prim[-1] / np.pi) * np.exp(-prim[-1] * ((u - prim[1]) ** 2 + (v - prim[2]) ** 2))


def sound_speed(lam, gamma):
    """src/Theory/theory_macro.jl:421-426"""
    return (0.5 * gamma / lam) ** 0.5


# ------------------------------------------------------------------ phase


def newton_cotes(idx, num):
    """Newton-Cotes weight coefficient of 1-based point idx out of num."""
    if idx == 1 or idx == num:
        return 14.0 / 45.0
    if (idx - 5) % 4 == 0:
        return 28.0 / 45.0
    if (idx - 3) % 4 == 0:
        return 24.0 / 45.0
    return 64.0 / 45.0


@dataclass
class VSpace1D:
    u0: float
    u1: float
    nu: int
    u: np.ndarray
    du: np.ndarray
    weights: np.ndarray

    @classmethod
    def build(cls, U0, U1, NU, type="rectangle"):
        d = (U1 - U0) / NU
        u = np.array([U0 + (i - 0.5) * d for i in range(1, NU + 1)], dtype=np.float64)
        if type == "rectangle":
            w = np.full(NU, d)
        elif type == "newton":
            w = np.array([newton_cotes(i, NU) * d for i in range(1, NU + 1)])
        else:
            raise ValueError("No velocity quadrature available: %r" % type)
        return cls(U0, U1, NU, u, np.full(NU, d), w)


@dataclass
class VSpace2D:
    u0: float
    u1: float
    nu: int
    v0: float
    v1: float
    nv: int
    u: np.ndarray  # (nu, nv), u index first like the reference
    v: np.ndarray
    du: np.ndarray
    dv: np.ndarray
    weights: np.ndarray

    @classmethod
    def build(cls, U0, U1, NU, V0, V1, NV, type="rectangle"):
        du, dv = (U1 - U0) / NU, (V1 - V0) / NV
        ui = np.array([U0 + (i - 0.5) * du for i in range(1, NU + 1)])
        vj = np.array([V0 + (j - 0.5) * dv for j in range(1, NV + 1)])
        u = np.repeat(ui[:, None], NV, axis=1)
        v = np.repeat(vj[None, :], NU, axis=0)
        if type == "rectangle":
            w = np.full((NU, NV), du * dv)
        elif type == "newton":
            cu = np.array([newton_cotes(i, NU) for i in range(1, NU + 1)])
            cv = np.array([newton_cotes(j, NV) for j in range(1, NV + 1)])
            # ((c_i * du) * c_j) * dv, evaluated in the reference's order
            w = ((cu[:, None] * du) * cv[None, :]) * dv
        else:
            raise ValueError("No velocity quadrature available: %r" % type)
        return cls(U0, U1, NU, V0, V1, NV, u, v, np.full((NU, NV), du), np.full((NU, NV), dv), w)

    def flat(self, a):
        """Column-major flattening (v = iu + nu * iv), the device order."""
        return np.ascontiguousarray(np.asarray(a).ravel(order="F"))


@dataclass
class PSpace1D:
    x0: float
    x1: float
    nx: int
    ng: int
    x: np.ndarray   # cell centres for i = 1-ng .. nx+ng (array index i-1+ng)
    dx: np.ndarray

    @classmethod
    def build(cls, X0, X1, NX, NG=0):
        d = (X1 - X0) / NX
        x = np.array([X0 + (i - 0.5) * d for i in range(1 - NG, NX + NG + 1)])
        return cls(X0, X1, NX, NG, x, np.full(NX + 2 * NG, d))


@dataclass
class PSpace2D:
    x0: float
    x1: float
    nx: int
    y0: float
    y1: float
    ny: int
    ngx: int
    ngy: int
    x: np.ndarray   # (nx+2ngx, ny+2ngy)
    y: np.ndarray
    dx: np.ndarray
    dy: np.ndarray

    @classmethod
    def build(cls, X0, X1, NX, Y0, Y1, NY, NGX=0, NGY=0):
        dx, dy = (X1 - X0) / NX, (Y1 - Y0) / NY
        xi = np.array([X0 + (i - 0.5) * dx for i in range(1 - NGX, NX + NGX + 1)])
        yj = np.array([Y0 + (j - 0.5) * dy for j in range(1 - NGY, NY + NGY + 1)])
        x = np.repeat(xi[:, None], len(yj), axis=1)
        y = np.repeat(yj[None, :], len(xi), axis=0)
        return cls(X0, X1, NX, Y0, Y1, NY, NGX, NGY, x, y, np.full_like(x, dx), np.full_like(x, dy))


# ---------------------------------------------------------------- config


def read_dict(filename):
    """`key = value` text with '#' comments; numbers parsed as Float64, kept as
    Int when integral, booleans recognised (src/IO/io_read.jl:95-128)."""
    out = {}
    with open(filename) as f:
        for line in f:
            line = line.rstrip("\n")
            if len(line) == 0 or line[0] == "#":
                continue
            if "=" not in line:
                continue
            var, val = line.split("=", 1)
            key = var.strip()
            val = val.split("#")[0]
            s = val.strip()
            try:
                x = float(s)
                out[key] = int(x) if x.is_integer() else x
            except ValueError:
                if s in ("true", "false"):
                    out[key] = s == "true"
                else:
                    out[key] = s
    return out


def read_cfg(filename):
    """src/IO/io_read.jl:12-43: expands `boundary` to one entry per side."""
    D = read_dict(filename)
    dim = int(D["space"][0])
    if "boundary" in D and isinstance(D["boundary"], str):
        D["boundary"] = [D["boundary"]] * (2 * dim)
    elif "boundary4" in D:
        D["boundary"] = [D["boundary1"], D["boundary2"], D["boundary3"], D["boundary4"]]
    elif "boundary2" in D:
        D["boundary"] = ([D["boundary1"], D["boundary2"]] if dim == 1 else
                         [D["boundary1"], D["boundary1"], D["boundary2"], D["boundary2"]])
    return D


@dataclass
class Setup:
    matter: str = "gas"
    case: str = "dev"
    space: str = "1d2f1v"
    flux: str = "kfvs"
    collision: str = "bgk"
    nSpecies: int = 1
    interpOrder: int = 2
    limiter: str = "vanleer"
    boundary: list = field(default_factory=lambda: ["fix", "fix"])
    cfl: float = 0.5
    maxTime: float = 0.1
    hasForce: bool = False


@dataclass
class Gas:
    Kn: float = 1e-2
    Ma: float = 0.0
    Pr: float = 1.0
    K: float = 2.0
    gamma: float = 5.0 / 3.0
    omega: float = 0.81
    alpha_ref: float = 1.0
    omega_ref: float = 0.5
    mu_ref: float = None

    def __post_init__(self):
        if self.mu_ref is None:
            self.mu_ref = ref_vhs_vis(self.Kn, self.alpha_ref, self.omega_ref)


def gas_property(space, inK, knudsen, mach=0.0, prandtl=1.0, omega=0.5, alphaRef=1.0,
                 omegaRef=0.5, nSpecies=1, **kw):
    """src/Struct/struct_property.jl:458-514 (single species, 2F)."""
    if nSpecies != 1:
        raise ValueError("only single-species gases are supported on the DVM path")
    D = int(space[0])
    gamma = heat_capacity_ratio(inK, D)
    return Gas(Kn=knudsen, Ma=mach, Pr=prandtl, K=inK, gamma=gamma, omega=omega,
               alpha_ref=alphaRef, omega_ref=omegaRef,
               mu_ref=ref_vhs_vis(knudsen, alphaRef, omegaRef))


# ------------------------------------------------------ initial conditions


@dataclass
class IB:
    """Initial / boundary condition: fw(x[, y]) -> w, bc(x[, y]) -> prim,
    ff -> (h, b) (the IB2F container of the reference)."""
    fw: object
    ff: object
    bc: object
    p: dict


def ib_sod(set_, ps, vs, gas):
    """ib_sod 1d2f1v (src/Config/cfg_sod.jl:6-62)."""
    primL, primR = np.array([1.0, 0.0, 0.5]), np.array([0.125, 0.0, 0.625])
    wL, wR = prim_conserve(primL, gas.gamma), prim_conserve(primR, gas.gamma)
    mid = (ps.x0 + ps.x1) / 2
    fw = lambda x: wL if x <= mid else wR
    bc = lambda x: primL if x <= mid else primR

    def ff(x):
        prim = conserve_prim(fw(x), gas.gamma)
        h = maxwellian(vs.u, prim)
        return h, h * gas.K / 2 / prim[-1]

    return IB(fw, ff, bc, dict(primL=primL, primR=primR, wL=wL, wR=wR))


def rh_states(Ma, gamma, lamL=1.0):
    """Upstream / downstream primitive states of a normal shock
    (src/Config/cfg_rh.jl:13-27).  The reference fixes the upstream
    lambda at 1; lamL generalises it with U = Ma sqrt(gamma / (2 lambda))."""
    MaR = math.sqrt((Ma ** 2 * (gamma - 1.0) + 2.0) / (2.0 * gamma * Ma ** 2 - (gamma - 1.0)))
    ratioT = ((1.0 + (gamma - 1.0) / 2.0 * Ma ** 2) * (2.0 * gamma / (gamma - 1.0) * Ma ** 2 - 1.0) /
              (Ma ** 2 * (2.0 * gamma / (gamma - 1.0) + (gamma - 1.0) / 2.0)))
    if lamL == 1.0:
        primL = np.array([1.0, Ma * math.sqrt(gamma / 2.0), 1.0])
        primR = np.array([primL[0] * (gamma + 1.0) * Ma ** 2 / ((gamma - 1.0) * Ma ** 2 + 2.0),
                          MaR * math.sqrt(gamma / 2.0) * math.sqrt(ratioT),
                          primL[2] / ratioT])
    else:
        primL = np.array([1.0, Ma * math.sqrt(gamma / (2.0 * lamL)), lamL])
        primR = np.array([primL[0] * (gamma + 1.0) * Ma ** 2 / ((gamma - 1.0) * Ma ** 2 + 2.0),
                          MaR * math.sqrt(gamma / (2.0 * lamL)) * math.sqrt(ratioT),
                          primL[2] / ratioT])
    return primL, primR


def ib_rh(set_, ps, vs, gas, lamL=1.0):
    """ib_rh 1d2f1v (src/Config/cfg_rh.jl:6-73)."""
    primL, primR = rh_states(gas.Ma, gas.gamma, lamL)
    wL, wR = prim_conserve(primL, gas.gamma), prim_conserve(primR, gas.gamma)
    mid = (ps.x0 + ps.x1) / 2
    fw = lambda x: wL if x <= mid else wR
    bc = lambda x: primL if x <= mid else primR

    def ff(x):
        prim = conserve_prim(fw(x), gas.gamma)
        h = maxwellian(vs.u, prim)
        return h, h * gas.K / 2 / prim[-1]

    return IB(fw, ff, bc, dict(primL=primL, primR=primR, wL=wL, wR=wR))


def ib_cavity(set_, ps, vs, gas, Um=0.15, Vm=0.0, Tm=1.0):
    """ib_cavity 2d2f2v (src/Config/cfg_cavity.jl:6-62).  The lid state is
    returned only where y == y1 exactly, as in the reference."""
    prim = np.array([1.0, 0.0, 0.0, 1.0])
    w = prim_conserve(prim, gas.gamma)
    primU = np.array([1.0, Um, Vm, Tm])
    h = maxwellian(vs.u, prim, vs.v)
    b = h * gas.K / 2.0 / prim[-1]
    fw = lambda x, y: w
    bc = lambda x, y: primU if y == ps.y1 else prim
    ff = lambda x, y: (h, b)
    return IB(fw, ff, bc, dict(prim=prim, primU=primU, w=w))


def ib_quadrant(set_, ps, vs, gas, seed=20261203, ranges=None):
    """Four-quadrant 2D Riemann-type state (no reference preset): prim
    [rho, U, V, lambda] per quadrant drawn from rho~U(0.1,1.5),
    U,V~U(-0.5,0.5), lambda~U(0.4,1.2) with a fixed seed, quadrants in the
    order (x>mid,y>mid), (x<=mid,y>mid), (x<=mid,y<=mid), (x>mid,y<=mid)."""
    rng = np.random.default_rng(seed)
    r = ranges or dict(rho=(0.1, 1.5), U=(-0.5, 0.5), V=(-0.5, 0.5), lam=(0.4, 1.2))
    quads = []
    for _ in range(4):
        quads.append(np.array([rng.uniform(*r["rho"]), rng.uniform(*r["U"]),
                               rng.uniform(*r["V"]), rng.uniform(*r["lam"])]))
    xm, ym = (ps.x0 + ps.x1) / 2, (ps.y0 + ps.y1) / 2

    def q(x, y):
        if x > xm and y > ym:
            return 0
        if x <= xm and y > ym:
            return 1
        if x <= xm and y <= ym:
            return 2
        return 3

    ws = [prim_conserve(p, gas.gamma) for p in quads]
    hs = []
    for p in quads:
        pp = conserve_prim(prim_conserve(p, gas.gamma), gas.gamma)
        h = maxwellian(vs.u, pp, vs.v)
        hs.append((h, h * gas.K / 2.0 / pp[-1]))
    fw = lambda x, y: ws[q(x, y)]
    bc = lambda x, y: quads[q(x, y)]
    ff = lambda x, y: hs[q(x, y)]
    return IB(fw, ff, bc, dict(quads=quads, seed=seed))


def config_ib(set_, ps, vs, gas, **kw):
    """src/Config/config.jl:16-28"""
    case = set_.case
    if case in ("shock", "rh"):
        return ib_rh(set_, ps, vs, gas, **kw)
    if case == "sod":
        return ib_sod(set_, ps, vs, gas)
    if case == "cavity":
        return ib_cavity(set_, ps, vs, gas, **kw)
    if case == "quadrant":
        return ib_quadrant(set_, ps, vs, gas, **kw)
    raise ValueError("no initial condition preset for case %r on the DVM path" % case)


# ------------------------------------------------------------- SolverSet


@dataclass
class SolverSet:
    set: Setup
    ps: object
    vs: object
    gas: Gas
    ib: IB
    config: dict = None  # the key/value configuration the set was built from
    ib_kw: dict = None   # keyword overrides of the initial-condition preset

    @property
    def dim(self):
        return int(self.set.space[0])

    @property
    def nf(self):
        """Distributions per cell: 1 for the 1F models (f), 2 for 2F (h, b)."""
        return int(self.set.space[2])


def solver_set(config, **ib_kw):
    """SolverSet(file or dict) (src/Solver/solver_set.jl:73-117) without the
    output-folder side effect."""
    D = read_cfg(config) if isinstance(config, str) else dict(config)
    space = D["space"]
    if space not in ("1d2f1v", "2d2f2v", "1d1f1v", "2d1f2v"):
        raise ValueError("the GPU DVM path covers 1d2f1v, 2d2f2v, 1d1f1v and 2d1f2v, not %r"
                         % space)
    dim = int(space[0])
    bc = D.get("boundary", ["fix"] * (2 * dim))
    if isinstance(bc, str):
        bc = [bc] * (2 * dim)
    s = Setup(matter=D.get("matter", "gas"), case=D.get("case", "dev"), space=space,
              flux=D.get("flux", "kfvs"), collision=D.get("collision", "bgk"),
              nSpecies=D.get("nSpecies", 1), interpOrder=D.get("interpOrder", 2),
              limiter=D.get("limiter", "vanleer"), boundary=list(bc),
              cfl=D.get("cfl", 0.5), maxTime=D.get("maxTime", 0.1),
              hasForce=D.get("hasForce", False))
    if s.limiter != "vanleer" and s.interpOrder == 2:
        raise ValueError("only the van Leer limiter is on the GPU DVM path")
    vtype = D.get("vMeshType", "rectangle")
    if dim == 1:
        ps = PSpace1D.build(D["x0"], D["x1"], D["nx"], D.get("nxg", 0))
        vs = VSpace1D.build(D["umin"], D["umax"], D["nu"], type=vtype)
    else:
        ps = PSpace2D.build(D["x0"], D["x1"], D["nx"], D["y0"], D["y1"], D["ny"],
                            D.get("nxg", 0), D.get("nyg", 0))
        vs = VSpace2D.build(D["umin"], D["umax"], D["nu"], D["vmin"], D["vmax"], D["nv"], type=vtype)
    gas = gas_property(space=space, inK=D["inK"], knudsen=D["knudsen"], mach=D.get("mach", 0.0),
                       prandtl=D.get("prandtl", 1.0), omega=D.get("omega", 0.5),
                       alphaRef=D.get("alphaRef", 1.0), omegaRef=D.get("omegaRef", 0.5),
                       nSpecies=D.get("nSpecies", 1))
    kw = dict(ib_kw)
    if s.case == "cavity" and "uLid" in D:
        kw.update(Um=D["uLid"], Vm=D["vLid"], Tm=D["tLid"])
    ib = config_ib(s, ps, vs, gas, **kw)
    return SolverSet(s, ps, vs, gas, ib, D, dict(ib_kw))
