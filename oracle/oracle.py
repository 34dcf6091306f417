"""TEST INFRASTRUCTURE ONLY: ctypes access to the FP64 CPU oracle (kb_oracle.c).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm
may import this module.  The product (kitbase.jl_gb300/kitgpu) never does.

PARITY UNPINNED: the reference (KitBase.jl, Julia) cannot run here and holds no
golden vectors for the DVM step; the oracle is pinned by invariants and known
answers in tests/test_oracle.py.

Besides the ctypes wrapper this file restates, independently of the product's
host code, the setup inputs the reference builds on the host: velocity grids
(src/Phase/phase_velocity.jl:14-65, :128-258; newton_cotes
src/Phase/phase_quadrature.jl:276-288) and the Sod / cavity initial states
(src/Config/cfg_sod.jl:52-62, src/Config/cfg_cavity.jl:6-62).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libkb_oracle.so")

FLUX = {"kfvs": 0, "kcu": 1, "ugks": 2}
COLL = {"bgk": 0, "shakhov": 1}
BC = {"fix": 0, "extra": 1, "period": 2, "maxwell": 3}


class KbConfig(ctypes.Structure):
    """Mirror of kb_config_t (include/kitgpu.h)."""

    _fields_ = [
        ("dim", ctypes.c_int32), ("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
        ("ngx", ctypes.c_int32), ("ngy", ctypes.c_int32),
        ("nu", ctypes.c_int32), ("nv", ctypes.c_int32),
        ("flux", ctypes.c_int32), ("collision", ctypes.c_int32),
        ("bc", ctypes.c_int32 * 4), ("interp_order", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("x0", ctypes.c_double), ("x1", ctypes.c_double),
        ("y0", ctypes.c_double), ("y1", ctypes.c_double),
        ("umax", ctypes.c_double), ("vmax", ctypes.c_double),
        ("K", ctypes.c_double), ("gamma", ctypes.c_double), ("mu_ref", ctypes.c_double),
        ("omega", ctypes.c_double), ("Pr", ctypes.c_double),
        ("nf", ctypes.c_int32),
    ]


def build(force=False):
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    if force or not os.path.exists(LIB):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


_lib = None
_D = ctypes.POINTER(ctypes.c_double)


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.kbo_create.restype = ctypes.c_void_p
        L.kbo_create.argtypes = [ctypes.POINTER(KbConfig), _D, _D, _D]
        L.kbo_destroy.argtypes = [ctypes.c_void_p]
        L.kbo_set_wall.argtypes = [ctypes.c_void_p, ctypes.c_int, _D]
        L.kbo_set_state.argtypes = [ctypes.c_void_p, _D, _D, _D, _D]
        L.kbo_get_state.argtypes = [ctypes.c_void_p, _D, _D, _D, _D]
        L.kbo_timestep.restype = ctypes.c_double
        L.kbo_timestep.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.kbo_reconstruct.argtypes = [ctypes.c_void_p]
        L.kbo_evolve.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.kbo_update.argtypes = [ctypes.c_void_p, ctypes.c_double, _D]
        L.kbo_step.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, _D]
        L.kbo_get_faces.argtypes = [ctypes.c_void_p, _D, _D, _D]
        L.kbo_get_slopes.argtypes = [ctypes.c_void_p, _D, _D, _D]
        L.kbo_set_threads.argtypes = [ctypes.c_int]
        L.kbo_max_threads.restype = ctypes.c_int
        L.kbo_gauss_moments.argtypes = [_D, ctypes.c_int, ctypes.c_double, _D, _D, _D, _D, _D]
        L.kbo_conserve_prim.argtypes = [_D, ctypes.c_int, ctypes.c_double, _D]
        L.kbo_prim_conserve.argtypes = [_D, ctypes.c_int, ctypes.c_double, _D]
        L.kbo_pdf_slope.argtypes = [_D, _D, ctypes.c_int, ctypes.c_double, _D]
        L.kbo_vanleer.restype = ctypes.c_double
        L.kbo_vanleer.argtypes = [ctypes.c_double, ctypes.c_double]
        L.kbo_psum.restype = ctypes.c_double
        L.kbo_psum.argtypes = [_D, ctypes.c_long]
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_D)


def make_config(dim, nx, ny, ngx, ngy, nu, nv, flux, collision, bc, interp_order, x0, x1, y0,
                y1, umax, vmax, K, gamma, mu_ref, omega, Pr, precision=0, nf=2):
    c = KbConfig()
    c.dim, c.nx, c.ny, c.ngx, c.ngy, c.nu, c.nv = dim, nx, ny, ngx, ngy, nu, nv
    c.flux = FLUX[flux] if isinstance(flux, str) else flux
    c.collision = COLL[collision] if isinstance(collision, str) else collision
    bcs = [bc] * 4 if isinstance(bc, (str, int)) else list(bc) + ["fix"] * (4 - len(bc))
    for k in range(4):
        c.bc[k] = BC[bcs[k]] if isinstance(bcs[k], str) else bcs[k]
    c.interp_order, c.precision = interp_order, precision
    c.x0, c.x1, c.y0, c.y1 = x0, x1, y0, y1
    c.umax, c.vmax = umax, vmax
    c.K, c.gamma, c.mu_ref, c.omega, c.Pr = K, gamma, mu_ref, omega, Pr
    c.nf = nf
    return c


class Oracle:
    """One oracle solver: same state layout as the C ABI (include/kitgpu.h)."""

    def __init__(self, cfg, u, v, weights, threads=None):
        self.L = lib()
        if threads is not None:
            self.L.kbo_set_threads(int(threads))
        self.cfg = cfg
        self.dim = cfg.dim
        self.nw = cfg.dim + 2
        nxt = cfg.nx + 2 * cfg.ngx
        nyt = cfg.ny + 2 * cfg.ngy if cfg.dim == 2 else 1
        self.ncell = nxt * nyt
        self.nvel = cfg.nu * (cfg.nv if cfg.dim == 2 else 1)
        self.nface = (cfg.nx + 1) * (cfg.ny if cfg.dim == 2 else 1) + (
            cfg.nx * (cfg.ny + 1) if cfg.dim == 2 else 0)
        self._u = np.ascontiguousarray(u, dtype=np.float64).ravel(order="F")
        self._v = np.ascontiguousarray(v if v is not None else np.zeros_like(self._u),
                                       dtype=np.float64).ravel(order="F")
        self._w = np.ascontiguousarray(weights, dtype=np.float64).ravel(order="F")
        self.h = self.L.kbo_create(ctypes.byref(cfg), _p(self._u), _p(self._v), _p(self._w))

    def __del__(self):
        if getattr(self, "h", None):
            self.L.kbo_destroy(self.h)
            self.h = None

    def set_wall(self, side, prim):
        prim = np.ascontiguousarray(prim, dtype=np.float64)
        self.L.kbo_set_wall(self.h, side, _p(prim))

    def set_state(self, w, prim, h, b):
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (w, prim, h, b)]
        self.L.kbo_set_state(self.h, *[_p(x) for x in a])

    def get_state(self):
        w = np.zeros((self.ncell, self.nw))
        prim = np.zeros_like(w)
        h = np.zeros((self.ncell, self.nvel))
        b = np.zeros_like(h)
        self.L.kbo_get_state(self.h, _p(w), _p(prim), _p(h), _p(b))
        return w, prim, h, b

    def timestep(self, cfl, t, tmax):
        return self.L.kbo_timestep(self.h, cfl, t, tmax)

    def reconstruct(self):
        self.L.kbo_reconstruct(self.h)

    def evolve(self, dt):
        self.L.kbo_evolve(self.h, dt)

    def update(self, dt):
        r = np.zeros(4)
        self.L.kbo_update(self.h, dt, _p(r))
        return r[: self.nw]

    def step(self, dt, n=1):
        r = np.zeros(4)
        self.L.kbo_step(self.h, dt, int(n), _p(r))
        return r[: self.nw]

    def faces(self):
        fw = np.zeros((self.nface, self.nw))
        fh = np.zeros((self.nface, self.nvel))
        fb = np.zeros_like(fh)
        self.L.kbo_get_faces(self.h, _p(fw), _p(fh), _p(fb))
        return fw, fh, fb

    def slopes(self):
        sw = np.zeros((self.ncell, self.dim, self.nw))
        sh = np.zeros((self.ncell, self.dim, self.nvel))
        sb = np.zeros_like(sh)
        self.L.kbo_get_slopes(self.h, _p(sw), _p(sh), _p(sb))
        return sw, sh, sb


# ---------------------------------------------------------------- pointwise

def gauss_moments(prim, inK):
    prim = np.ascontiguousarray(prim, dtype=np.float64)
    Mu, Mv, MuL, MuR = (np.zeros(7) for _ in range(4))
    Mxi = np.zeros(3)
    lib().kbo_gauss_moments(_p(prim), len(prim), float(inK), _p(Mu), _p(Mv), _p(Mxi), _p(MuL), _p(MuR))
    return Mu, Mv, Mxi, MuL, MuR


def conserve_prim(w, gamma):
    w = np.ascontiguousarray(w, dtype=np.float64)
    p = np.zeros_like(w)
    lib().kbo_conserve_prim(_p(w), len(w), float(gamma), _p(p))
    return p


def prim_conserve(prim, gamma):
    prim = np.ascontiguousarray(prim, dtype=np.float64)
    w = np.zeros_like(prim)
    lib().kbo_prim_conserve(_p(prim), len(prim), float(gamma), _p(w))
    return w


def pdf_slope(prim, sw, inK):
    prim = np.ascontiguousarray(prim, dtype=np.float64)
    sw = np.ascontiguousarray(sw, dtype=np.float64)
    sl = np.zeros_like(prim)
    lib().kbo_pdf_slope(_p(prim), _p(sw), len(prim), float(inK), _p(sl))
    return sl


def vanleer(sL, sR):
    return lib().kbo_vanleer(float(sL), float(sR))


def psum(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return lib().kbo_psum(_p(a), a.size)


# ------------------------------------------------- independent setup inputs

def newton_cotes(idx, num):
    """src/Phase/phase_quadrature.jl:276-288 (1-based idx)."""
    if idx == 1 or idx == num:
        return 14.0 / 45.0
    if (idx - 5) % 4 == 0:
        return 28.0 / 45.0
    if (idx - 3) % 4 == 0:
        return 24.0 / 45.0
    return 64.0 / 45.0


def vspace1d(u0, u1, nu, mesh="newton"):
    d = (u1 - u0) / nu
    u = np.array([u0 + (i - 0.5) * d for i in range(1, nu + 1)])
    if mesh == "newton":
        w = np.array([newton_cotes(i, nu) * d for i in range(1, nu + 1)])
    else:
        w = np.full(nu, d)
    return u, w


def vspace2d(u0, u1, nu, v0, v1, nv, mesh="newton"):
    """Returns flat arrays in column-major (u fastest) order."""
    du, dv = (u1 - u0) / nu, (v1 - v0) / nv
    U = np.zeros((nu, nv)); V = np.zeros((nu, nv)); W = np.zeros((nu, nv))
    for j in range(1, nv + 1):
        for i in range(1, nu + 1):
            U[i - 1, j - 1] = u0 + (i - 0.5) * du
            V[i - 1, j - 1] = v0 + (j - 0.5) * dv
            if mesh == "newton":
                W[i - 1, j - 1] = newton_cotes(i, nu) * du * newton_cotes(j, nv) * dv
            else:
                W[i - 1, j - 1] = du * dv
    return U.ravel(order="F"), V.ravel(order="F"), W.ravel(order="F")


def maxwellian1(u, prim):
    """src/Theory/theory_equilibrium.jl:8-13"""
    return prim[0] * np.sqrt(prim[-1] / np.pi) * np.exp(-prim[-1] * (u - prim[1]) ** 2)


def maxwellian2(u, v, prim):
    """src/Theory/theory_equilibrium.jl:20-25"""
    return prim[0] * (prim[-1] / np.pi) * np.exp(-prim[-1] * ((u - prim[1]) ** 2 + (v - prim[2]) ** 2))


def sod_state(nx, ng, x0, x1, u, gamma, K):
    """ib_sod 1d2f1v (src/Config/cfg_sod.jl:6-62) on PSpace1D(x0, x1, nx, ng)."""
    d = (x1 - x0) / nx
    wL = prim_conserve([1.0, 0.0, 0.5], gamma)
    wR = prim_conserve([0.125, 0.0, 0.625], gamma)
    ncell = nx + 2 * ng
    W = np.zeros((ncell, 3)); P = np.zeros((ncell, 3))
    H = np.zeros((ncell, len(u))); B = np.zeros_like(H)
    for c in range(ncell):
        i = c - ng + 1
        x = x0 + (i - 0.5) * d
        w = wL if x <= (x0 + x1) / 2 else wR
        p = conserve_prim(w, gamma)
        W[c], P[c] = w, p
        H[c] = maxwellian1(u, p)
        B[c] = H[c] * K / 2 / p[-1]
    return W, P, H, B


def cavity_state(nx, ny, ngx, ngy, u, v, gamma, K):
    """ib_cavity 2d2f2v (src/Config/cfg_cavity.jl:6-62): uniform [1, 0, 0, 1]."""
    prim = np.array([1.0, 0.0, 0.0, 1.0])
    w = prim_conserve(prim, gamma)
    p = conserve_prim(w, gamma)
    ncell = (nx + 2 * ngx) * (ny + 2 * ngy)
    h = maxwellian2(u, v, prim)
    b = h * K / 2.0 / prim[-1]
    return (np.tile(w, (ncell, 1)), np.tile(p, (ncell, 1)), np.tile(h, (ncell, 1)),
            np.tile(b, (ncell, 1)))


def cavity_walls(nx, ny, x0, x1, y0, y1, lid=(0.15, 0.0, 1.0)):
    """KS.ib.bc at the wall face midpoints (src/Solver/evolve_boundary.jl:52-178;
    lid test y == y1, src/Config/cfg_cavity.jl:30)."""
    dx, dy = (x1 - x0) / nx, (y1 - y0) / ny
    base = np.array([1.0, 0.0, 0.0, 1.0])
    top = np.array([1.0, lid[0], lid[1], lid[2]])
    walls = []
    for s in range(4):
        n = ny if s < 2 else nx
        arr = np.zeros((n, 4))
        for q in range(1, n + 1):
            if s < 2:
                y = y0 + (q - 0.5) * dy
                yc = ((y - 0.5 * dy) + (y + 0.5 * dy)) / 2
            elif s == 2:
                yc = y0 + (1 - 0.5) * dy - 0.5 * dy
            else:
                yc = y0 + (ny - 0.5) * dy + 0.5 * dy
            arr[q - 1] = top if yc == y1 else base
        walls.append(arr)
    return walls
