"""Batched ensembles of independent 1D2F1V solves (kb_batch_* in the C ABI).

All instances advance in one persistent kernel launch per step, two steps per
captured CUDA graph; each instance keeps its own cell count, velocity grid,
time step and convergence state, and stops (its state carried unchanged) once
its residual falls below the tolerance.  `shock_ensemble` draws the normal
shock-structure ensemble: Mach ~ U(1.2, 8), cells ~ U{50..400}, velocities
~ U{48..200} on +-(5 + 2 Ma), Rankine-Hugoniot states with upstream rho = 1,
lambda = 0.5, Shakhov relaxation at Kn = 1.
"""
import ctypes

import numpy as np

from . import _native as N
from .setup import rh_states, solver_set
from .solver import initial_state, kb_config

_BATCH_SIGS = {
    "kb_batch_create": [ctypes.POINTER(N.KbConfig), ctypes.c_int32] + [ctypes.POINTER(ctypes.c_int32)] * 3
    + [ctypes.POINTER(ctypes.c_double)] * 6 + [ctypes.POINTER(ctypes.c_void_p)],
    "kb_batch_destroy": [ctypes.c_void_p],
    "kb_batch_upload": [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_double)] * 4,
    "kb_batch_download": [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_double)] * 4,
    "kb_batch_init_equilibrium": [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_double)] * 2,
    "kb_batch_timestep": [ctypes.c_void_p, ctypes.c_double, ctypes.POINTER(ctypes.c_double)],
    "kb_batch_set_dt": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)],
    "kb_batch_step": [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double,
                      ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int32)],
    "kb_batch_info": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)],
    "kb_batch_set_tuning": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.c_int32],
    "kb_batch_get_tuning": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.c_int32],
}


def _lib():
    lib = N.load()
    for name, args in _BATCH_SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    return lib


def _i32(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def shock_config(Ma, nx, nu, Kn=1.0, lam_up=0.5, cfl=0.5, coll="shakhov"):
    """One normal-shock-structure instance (the reference's ib_rh preset with the
    upstream lambda generalised, src/Config/cfg_rh.jl:6-73)."""
    umax = 5.0 + 2.0 * Ma
    return dict(matter="gas", case="shock", space="1d2f1v", flux="kfvs", collision=coll,
                nSpecies=1, interpOrder=2, limiter="vanleer", boundary="fix", cfl=cfl,
                maxTime=1.0e9, x0=-35.0, x1=35.0, nx=int(nx), nxg=0, umin=-umax, umax=umax,
                nu=int(nu), vMeshType="rectangle", knudsen=Kn, mach=float(Ma), prandtl=2.0 / 3.0,
                inK=2.0, omega=0.72, alphaRef=1.0, omegaRef=0.5, _lam_up=lam_up)


def solver_sets(configs):
    out = []
    for cfg in configs:
        cfg = dict(cfg)
        lam = cfg.pop("_lam_up", 1.0)
        out.append(solver_set(cfg, lamL=lam) if cfg["case"] in ("shock", "rh") else solver_set(cfg))
    return out


def shock_ensemble(n=512, seed=20261203, Kn=1.0, coll="shakhov"):
    """Configs of the batched shock-structure ensemble."""
    rng = np.random.default_rng(seed)
    cfgs = []
    for _ in range(n):
        Ma = rng.uniform(1.2, 8.0)
        nx = int(rng.integers(50, 401))
        nu = int(rng.integers(48, 201))
        cfgs.append(shock_config(Ma, nx, nu, Kn=Kn, coll=coll))
    return cfgs


class Batch:
    """A batch of 1D solves resident on the GPU."""

    def __init__(self, solver_sets_list, precision="fp32"):
        self.lib = _lib()
        self.KS = list(solver_sets_list)
        if not self.KS:
            raise ValueError("empty batch")
        base = kb_config(self.KS[0], precision)
        self.prec = precision
        self.n = len(self.KS)
        nx = np.array([K.ps.nx for K in self.KS], dtype=np.int32)
        ng = np.array([K.ps.ng for K in self.KS], dtype=np.int32)
        nu = np.array([K.vs.nu for K in self.KS], dtype=np.int32)
        x0 = np.array([K.ps.x0 for K in self.KS], dtype=np.float64)
        x1 = np.array([K.ps.x1 for K in self.KS], dtype=np.float64)
        umax = np.array([K.vs.u1 for K in self.KS], dtype=np.float64)
        mu = np.array([K.gas.mu_ref for K in self.KS], dtype=np.float64)
        for K in self.KS:
            if (K.gas.K, K.gas.gamma, K.gas.omega, K.gas.Pr) != (base.K, base.gamma, base.omega, base.Pr):
                raise ValueError("all instances of a batch share K, gamma, omega and Pr")
            if K.set.collision != self.KS[0].set.collision or K.set.flux != "kfvs":
                raise ValueError("all instances of a batch share the collision model (KFVS flux)")
        u_all = np.concatenate([K.vs.u for K in self.KS])
        w_all = np.concatenate([K.vs.weights for K in self.KS])
        self.nx, self.ng, self.nu = nx, ng, nu
        self._keep = [_i32(nx), _i32(ng), _i32(nu), x0, x1, umax, mu, u_all, w_all]
        h = ctypes.c_void_p()
        N.check(self.lib.kb_batch_create(ctypes.byref(base), self.n, self._keep[0][1], self._keep[1][1],
                                         self._keep[2][1], N.ptr(x0), N.ptr(x1), N.ptr(umax),
                                         N.ptr(mu), N.ptr(u_all), N.ptr(w_all), ctypes.byref(h)))
        self.h = h
        self.ncells = nx + 2 * ng
        self.cell_off = np.concatenate([[0], np.cumsum(self.ncells)])
        self.elem_off = np.concatenate([[0], np.cumsum(self.ncells.astype(np.int64) * nu)])
        self.residual = np.zeros((self.n, 4))
        self.active = np.ones(self.n, dtype=np.int32)
        self.steps = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.kb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload_initial(self):
        parts = [initial_state(K) for K in self.KS]
        w = np.ascontiguousarray(np.concatenate([p[0] for p in parts]))
        p = np.ascontiguousarray(np.concatenate([p[1] for p in parts]))
        h = np.ascontiguousarray(np.concatenate([q[2].ravel() for q in parts]))
        b = np.ascontiguousarray(np.concatenate([q[3].ravel() for q in parts]))
        N.check(self.lib.kb_batch_upload(self.h, N.ptr(w), N.ptr(p), N.ptr(h), N.ptr(b)))
        self.active[:] = 1
        return w, p, h, b

    def init_initial(self):
        """init_fvm's equilibrium state of every instance, h and b built on
        the device (kb_batch_init_equilibrium): only w and prim cross the bus,
        and the FP32 split form starts from its own FP32 Maxwellian."""
        from .solver import initial_cells
        parts = [initial_cells(K) for K in self.KS]
        w = np.ascontiguousarray(np.concatenate([p[0] for p in parts]))
        p = np.ascontiguousarray(np.concatenate([p[1] for p in parts]))
        N.check(self.lib.kb_batch_init_equilibrium(self.h, N.ptr(w), N.ptr(p)))
        self.active[:] = 1
        return w, p

    def timestep(self):
        dt = np.zeros(self.n)
        N.check(self.lib.kb_batch_timestep(self.h, float(self.KS[0].set.cfl), N.ptr(dt)))
        self.dt = dt
        return dt

    def set_dt(self, dt):
        dt = np.ascontiguousarray(dt, dtype=np.float64)
        N.check(self.lib.kb_batch_set_dt(self.h, N.ptr(dt)))
        self.dt = dt

    def step(self, nsteps, tol=0.0):
        act = np.zeros(self.n, dtype=np.int32)
        N.check(self.lib.kb_batch_step(self.h, int(nsteps), float(tol), N.ptr(self.residual),
                                       act.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))))
        self.active = act
        self.steps += nsteps
        return self.residual[:, :3].copy()

    def run_to_steady(self, tol=1e-8, max_steps=20000, chunk=200):
        """Step until every instance's residual is below tol (or max_steps)."""
        while self.steps < max_steps and self.active.any():
            self.step(min(chunk, max_steps - self.steps), tol)
        return int(self.active.sum())

    def upload(self, states):
        """Per-instance states (dicts with w, prim, h, b as download() returns)."""
        w = np.ascontiguousarray(np.concatenate([x["w"] for x in states]))
        p = np.ascontiguousarray(np.concatenate([x["prim"] for x in states]))
        h = np.ascontiguousarray(np.concatenate([x["h"].ravel() for x in states]))
        b = np.ascontiguousarray(np.concatenate([x["b"].ravel() for x in states]))
        N.check(self.lib.kb_batch_upload(self.h, N.ptr(w), N.ptr(p), N.ptr(h), N.ptr(b)))
        self.active[:] = 1

    def download(self):
        ncell = int(self.cell_off[-1])
        nel = int(self.elem_off[-1])
        w = np.zeros((ncell, 3))
        p = np.zeros((ncell, 3))
        h = np.zeros(nel)
        b = np.zeros(nel)
        N.check(self.lib.kb_batch_download(self.h, N.ptr(w), N.ptr(p), N.ptr(h), N.ptr(b)))
        out = []
        for k in range(self.n):
            c0, c1 = self.cell_off[k], self.cell_off[k + 1]
            e0, e1 = self.elem_off[k], self.elem_off[k + 1]
            nuk = int(self.nu[k])
            out.append(dict(w=w[c0:c1], prim=p[c0:c1], h=h[e0:e1].reshape(-1, nuk),
                            b=b[e0:e1].reshape(-1, nuk)))
        return out

    def set_tuning(self, seg=16, threads=128, persist=0):
        """Shape of the FP32 step kernel: cells per segment, threads per CTA,
        persistent grid (kb_batch_set_tuning)."""
        arr = (ctypes.c_int32 * 3)(int(seg), int(threads), int(persist))
        N.check(self.lib.kb_batch_set_tuning(self.h, arr, 3))

    def tuning(self):
        arr = (ctypes.c_int32 * 3)()
        N.check(self.lib.kb_batch_get_tuning(self.h, arr, 3))
        return dict(seg=arr[0], threads=arr[1], persist=arr[2])

    def launches(self):
        e, l = ctypes.c_int64(), ctypes.c_int64()
        N.check(self.lib.kb_batch_info(self.h, ctypes.byref(e), ctypes.byref(l)))
        return l.value

    def cell_velocity_points(self):
        return int(np.sum(self.nx.astype(np.int64) * self.nu))


_POOL_SIGS = {
    "kb_pool_create": [ctypes.POINTER(N.KbConfig), ctypes.c_int32, ctypes.c_int64, ctypes.c_int32,
                       ctypes.POINTER(ctypes.c_void_p)],
    "kb_pool_add": [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                    ctypes.c_double, ctypes.c_double, ctypes.c_double] + [ctypes.POINTER(ctypes.c_double)] * 4
    + [ctypes.c_double, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_double)],
    "kb_pool_remove": [ctypes.c_void_p, ctypes.c_int32],
    "kb_pool_download": [ctypes.c_void_p, ctypes.c_int32] + [ctypes.POINTER(ctypes.c_double)] * 4,
}


def _pool_lib():
    lib = _lib()
    for name, args in _POOL_SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    return lib


def poolable(KS):
    """A solve the pool can hold: 1D2F1V, KFVS, fixed boundaries, van Leer,
    at most 256 velocities (the batch kernel's coverage)."""
    return (KS.dim == 1 and KS.nf == 2 and KS.set.flux == "kfvs" and KS.vs.nu <= 256
            and list(KS.set.boundary)[:2] == ["fix", "fix"] and KS.set.interpOrder == 2)


def pool_key(KS):
    """Gas constants and collision model a pool's instances share."""
    g = KS.gas
    return (g.K, g.gamma, g.omega, g.Pr, KS.set.collision)


class Pool:
    """Continuous batching of 1D solves (kb_pool_*): a resident FP32-split
    batch with fixed capacity that solves join (`add`) and leave (`remove`)
    between steps; `step` advances every resident solve with one fused launch
    per step (two steps per replayed CUDA graph)."""

    def __init__(self, base_KS, max_instances=64, max_cells=64 * 2052, max_nu=256):
        self.lib = _pool_lib()
        self.key = pool_key(base_KS)
        cfg = kb_config(base_KS, "fp32")
        self.n = int(max_instances)
        h = ctypes.c_void_p()
        N.check(self.lib.kb_pool_create(ctypes.byref(cfg), self.n, int(max_cells), int(max_nu),
                                        ctypes.byref(h)))
        self.h = h
        self.max_cells = int(max_cells)
        self.slots = {}  # slot -> KS
        self.residual = np.zeros((self.n, 4))
        self.active = np.zeros(self.n, dtype=np.int32)

    def close(self):
        if getattr(self, "h", None):
            self.lib.kb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, KS):
        """Place one solve (its init_fvm equilibrium state); returns (slot, dt)."""
        from .solver import initial_cells
        if pool_key(KS) != self.key or not poolable(KS):
            raise ValueError("this solve does not fit the pool")
        w, p = initial_cells(KS)
        w = np.ascontiguousarray(w, dtype=np.float64)
        p = np.ascontiguousarray(p, dtype=np.float64)
        u = np.ascontiguousarray(KS.vs.u, dtype=np.float64)
        wt = np.ascontiguousarray(KS.vs.weights, dtype=np.float64)
        slot, dt = ctypes.c_int32(), ctypes.c_double()
        N.check(self.lib.kb_pool_add(self.h, KS.ps.nx, KS.ps.ng, KS.vs.nu, KS.ps.x0, KS.ps.x1,
                                     KS.vs.u1, KS.gas.mu_ref, N.ptr(u), N.ptr(wt), N.ptr(w),
                                     N.ptr(p), float(KS.set.cfl), ctypes.byref(slot),
                                     ctypes.byref(dt)))
        self.slots[slot.value] = KS
        self.active[slot.value] = 1
        return slot.value, dt.value

    def remove(self, slot):
        N.check(self.lib.kb_pool_remove(self.h, int(slot)))
        self.slots.pop(int(slot), None)
        self.active[slot] = 0

    def download(self, slot, want=("w", "prim", "h", "b")):
        KS = self.slots[int(slot)]
        nc = KS.ps.nx + 2 * KS.ps.ng
        out = {k: (np.zeros((nc, 3)) if k in ("w", "prim") else np.zeros((nc, KS.vs.nu)))
               for k in want}
        N.check(self.lib.kb_pool_download(self.h, int(slot), N.ptr(out.get("w")),
                                          N.ptr(out.get("prim")), N.ptr(out.get("h")),
                                          N.ptr(out.get("b"))))
        return out

    def step(self, nsteps, tol=0.0):
        """nsteps steps of every resident solve; a solve whose residual falls
        below tol stops (state carried).  Returns the residuals [n][3]."""
        act = np.zeros(self.n, dtype=np.int32)
        N.check(self.lib.kb_batch_step(self.h, int(nsteps), float(tol), N.ptr(self.residual),
                                       act.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))))
        self.active = act
        return self.residual[:, :3]

    def set_tuning(self, seg=16, threads=128, persist=1):
        arr = (ctypes.c_int32 * 3)(int(seg), int(threads), int(persist))
        N.check(self.lib.kb_batch_set_tuning(self.h, arr, 3))

    def launches(self):
        e, l = ctypes.c_int64(), ctypes.c_int64()
        N.check(self.lib.kb_batch_info(self.h, ctypes.byref(e), ctypes.byref(l)))
        return l.value
