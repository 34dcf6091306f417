"""Device-resident drop-in for KitBase's DVM solver path.

The reference keeps an OffsetArray of ControlVolume2F cells and arrays of
Interface2F faces on the host and advances them with reconstruct!, evolve!
and update! (src/Solver/solver_reconstruction.jl, solver_evolution.jl,
solver_update.jl) inside solve! (src/Solver/solver_main.jl:12-150).  Here
the cells and faces live in HBM behind a libkitgpu handle; `Cells` and
`Faces` are views that download on access, and the stage functions keep the
reference's names (without the `!`), argument order and keyword meaning.
"""
import ctypes
import json
import math
from collections import namedtuple

import numpy as np

from . import _native as N
from .setup import conserve_prim, read_dict, solver_set

ControlVolume = namedtuple("ControlVolume", "w prim h b")


def kb_config(KS, precision="fp64"):
    """kb_config_t from a SolverSet."""
    s, ps, vs, gas = KS.set, KS.ps, KS.vs, KS.gas
    D = KS.dim
    c = N.KbConfig()
    c.dim = D
    c.nx = ps.nx
    c.ny = ps.ny if D == 2 else 1
    c.ngx = ps.ng if D == 1 else ps.ngx
    c.ngy = ps.ngy if D == 2 else 0
    c.nu = vs.nu
    c.nv = vs.nv if D == 2 else 1
    if s.flux not in N.FLUX:
        raise ValueError("flux %r is not on the GPU DVM path" % s.flux)
    if s.collision not in N.COLLISION:
        raise ValueError("collision %r is not on the GPU DVM path" % s.collision)
    c.flux = N.FLUX[s.flux]
    c.collision = N.COLLISION[s.collision]
    bc = list(s.boundary) + ["fix"] * (4 - len(s.boundary))
    for k in range(4):
        if bc[k] not in N.BOUNDARY:
            raise ValueError("boundary %r is not on the GPU DVM path" % bc[k])
        c.bc[k] = N.BOUNDARY[bc[k]]
    c.interp_order = s.interpOrder
    c.precision = N.PRECISION[precision]
    c.x0, c.x1 = ps.x0, ps.x1
    c.y0, c.y1 = (ps.y0, ps.y1) if D == 2 else (0.0, 1.0)
    c.umax = vs.u1
    c.vmax = vs.v1 if D == 2 else 0.0
    c.K, c.gamma, c.mu_ref, c.omega, c.Pr = gas.K, gas.gamma, gas.mu_ref, gas.omega, gas.Pr
    c.nf = KS.nf
    return c


class Handle:
    """Owner of one kb_handle_t."""

    def __init__(self, cfg, u, v, weights):
        self.lib = N.load()
        self.cfg = cfg
        self.dim = cfg.dim
        self.nw = cfg.dim + 2
        self.nxt = cfg.nx + 2 * cfg.ngx
        self.nyt = cfg.ny + 2 * cfg.ngy if cfg.dim == 2 else 1
        self.ncell = self.nxt * self.nyt
        self.nvel = cfg.nu * (cfg.nv if cfg.dim == 2 else 1)
        self.nface = (cfg.nx + 1) * (cfg.ny if cfg.dim == 2 else 1) + (
            cfg.nx * (cfg.ny + 1) if cfg.dim == 2 else 0)
        self._u = np.ascontiguousarray(u, dtype=np.float64).ravel()
        self._v = None if v is None else np.ascontiguousarray(v, dtype=np.float64).ravel()
        self._w = np.ascontiguousarray(weights, dtype=np.float64).ravel()
        h = N._H()
        N.check(self.lib.kb_create(ctypes.byref(cfg), N.ptr(self._u), N.ptr(self._v),
                                   N.ptr(self._w), ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.kb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def call(self, name, *args):
        return N.check(getattr(self.lib, name)(self.h, *args))

    def upload(self, w, prim, h, b=None):
        """Cell state host -> device; b may be None for the 1F models."""
        a = [None if x is None else np.ascontiguousarray(x, dtype=np.float64)
             for x in (w, prim, h, b)]
        self.call("kb_upload_state", *[N.ptr(x) for x in a])

    def init_equilibrium(self, w, prim):
        """w, prim per cell; h, b set to the equilibrium on the device."""
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (w, prim)]
        self.call("kb_init_equilibrium", *[N.ptr(x) for x in a])

    def download(self, want=("w", "prim", "h", "b")):
        out = {}
        w = np.zeros((self.ncell, self.nw)) if "w" in want else None
        p = np.zeros((self.ncell, self.nw)) if "prim" in want else None
        h = np.zeros((self.ncell, self.nvel)) if "h" in want else None
        b = np.zeros((self.ncell, self.nvel)) if "b" in want else None
        self.call("kb_download_state", N.ptr(w), N.ptr(p), N.ptr(h), N.ptr(b))
        for k, a in zip(("w", "prim", "h", "b"), (w, p, h, b)):
            if a is not None:
                out[k] = a
        return out

    def set_wall(self, side, prim):
        prim = np.ascontiguousarray(prim, dtype=np.float64)
        self.call("kb_set_wall", int(side), N.ptr(prim))

    def timestep(self, cfl, t, tmax):
        dt = ctypes.c_double()
        self.call("kb_timestep", float(cfl), float(t), float(tmax), ctypes.byref(dt))
        return dt.value

    def reconstruct(self):
        self.call("kb_reconstruct")

    def evolve(self, dt):
        self.call("kb_evolve", float(dt))

    def update(self, dt):
        r = np.zeros(4)
        self.call("kb_update", float(dt), N.ptr(r))
        return r[: self.nw]

    def step_cfl(self, cfl, t, max_time, n=1):
        """n steps, each with dt recomputed from the current state on the
        device (kb_step_cfl); returns (time reached, last residual)."""
        r = np.zeros(4)
        to = ctypes.c_double()
        self.call("kb_step_cfl", float(cfl), float(t), float(max_time), int(n), ctypes.byref(to), N.ptr(r))
        return to.value, r[: self.nw]

    def step(self, dt, n=1):
        r = np.zeros(4)
        self.call("kb_step", float(dt), int(n), N.ptr(r))
        return r[: self.nw]

    def step_async(self, dt, n=1):
        self.call("kb_step_async", float(dt), int(n))

    def query(self):
        """(ready, residual) of the last step_async."""
        r = np.zeros(4)
        ready = ctypes.c_int32()
        self.call("kb_query", N.ptr(r), ctypes.byref(ready))
        return bool(ready.value), r[: self.nw]

    def faces(self, dt):
        fw = np.zeros((self.nface, self.nw))
        fh = np.zeros((self.nface, self.nvel))
        fb = np.zeros_like(fh)
        self.call("kb_download_faces", float(dt), N.ptr(fw), N.ptr(fh), N.ptr(fb))
        return fw, fh, fb

    def upload_slopes(self, sw):
        """w slopes [ncell, dim, dim+2] (ctr.sw), e.g. from a checkpoint."""
        sw = np.ascontiguousarray(sw, dtype=np.float64)
        if sw.shape != (self.ncell, self.dim, self.nw):
            raise ValueError("sw has shape %s, expected %s" % (sw.shape, (self.ncell, self.dim, self.nw)))
        self.call("kb_upload_slopes", N.ptr(sw))

    def slopes(self):
        sw = np.zeros((self.ncell, self.dim, self.nw))
        sh = np.zeros((self.ncell, self.dim, self.nvel))
        sb = np.zeros_like(sh)
        self.call("kb_download_slopes", N.ptr(sw), N.ptr(sh), N.ptr(sb))
        return sw, sh, sb

    def status(self):
        return self.lib.kb_status(self.h)

    def launches(self):
        n = ctypes.c_int64()
        self.call("kb_launch_count", ctypes.byref(n))
        return n.value

    def set_timing(self, on=True):
        self.call("kb_set_timing", 1 if on else 0)

    def timing(self):
        ms = np.zeros(len(N.STAGES))
        n = (ctypes.c_int64 * len(N.STAGES))()
        self.call("kb_get_timing", N.ptr(ms), n)
        return {k: (ms[i], n[i]) for i, k in enumerate(N.STAGES)}

    def set_tuning(self, march_tx=0, march_ry=0, march_bs=0, mom_ts=0):
        arr = (ctypes.c_int32 * 4)(march_tx, march_ry, march_bs, mom_ts)
        self.call("kb_set_tuning", arr, 4)

    def tuning(self):
        arr = (ctypes.c_int32 * 4)()
        self.call("kb_get_tuning", arr, 4)
        return dict(zip(("march_tx", "march_ry", "march_bs", "mom_ts"), list(arr)))

    def stream(self):
        p = ctypes.c_void_p()
        self.call("kb_get_stream", ctypes.byref(p))
        return p.value

    def device_bytes(self):
        n = ctypes.c_int64()
        self.call("kb_device_bytes", ctypes.byref(n))
        return n.value


class Cells:
    """Device-resident array of ControlVolume2F (1-based, ghosts at 1-ng..)."""

    def __init__(self, KS, handle):
        self.KS = KS
        self.handle = handle

    @property
    def dim(self):
        return self.handle.dim

    def _ci(self, i, j=1):
        c = self.handle.cfg
        return (j - 1 + c.ngy) * self.handle.nxt + (i - 1 + c.ngx)

    def state(self):
        return self.handle.download()

    def __getitem__(self, idx):
        i, j = (idx, 1) if not isinstance(idx, tuple) else idx
        s = self.handle.download()
        c = self._ci(i, j)
        h, b = s["h"][c], s["b"][c]
        if self.dim == 2:
            vs = self.KS.vs
            h = h.reshape((vs.nu, vs.nv), order="F")
            b = b.reshape((vs.nu, vs.nv), order="F")
        return ControlVolume(s["w"][c], s["prim"][c], h, b)


class Faces:
    """Face fluxes of the last evolve (Interface2F arrays), downloaded on access."""

    def __init__(self, handle, direction):
        self.handle = handle
        self.direction = direction
        self.dt = None

    def fluxes(self):
        if self.dt is None:
            raise RuntimeError("no evolve has run on these faces yet")
        fw, fh, fb = self.handle.faces(self.dt)
        nfx = (self.handle.cfg.nx + 1) * (self.handle.cfg.ny if self.handle.dim == 2 else 1)
        sl = slice(0, nfx) if self.direction == 0 else slice(nfx, None)
        return fw[sl], fh[sl], fb[sl]


def initial_cells(KS):
    """Per-cell (w, prim) of init_fvm, all cells incl. ghosts, x fastest."""
    ps, ib, gas = KS.ps, KS.ib, KS.gas
    if KS.dim == 1:
        pts = [(x,) for x in ps.x]
    else:
        nxt, nyt = ps.x.shape
        pts = [(ps.x[i, j], ps.y[i, j]) for j in range(nyt) for i in range(nxt)]
    ws, ps_ = [], []
    cache = {}
    for pt in pts:
        w = np.asarray(ib.fw(*pt), dtype=np.float64)
        key = w.tobytes()
        if key not in cache:
            cache[key] = conserve_prim(w, gas.gamma)
        ws.append(w)
        ps_.append(cache[key])
    return np.array(ws), np.array(ps_)


def initial_state(KS):
    """Per-cell (w, prim, h, b) of init_fvm (src/Solver/solver_init.jl:119-141,
    :285-325), all cells incl. ghosts, x fastest; flat velocity order.  For
    the 1F models h holds f and b is zero."""
    ps, ib, gas = KS.ps, KS.ib, KS.gas
    if KS.dim == 1:
        xs = list(ps.x)
        pts = [(x,) for x in xs]
    else:
        nxt, nyt = ps.x.shape
        pts = [(ps.x[i, j], ps.y[i, j]) for j in range(nyt) for i in range(nxt)]
    ws, ps_, hs, bs = [], [], [], []
    cache = {}
    for pt in pts:
        w = np.asarray(ib.fw(*pt), dtype=np.float64)
        key = w.tobytes()
        if key not in cache:
            h, b = ib.ff(*pt)
            if KS.dim == 2:
                h = np.asarray(h).ravel(order="F")
                b = np.asarray(b).ravel(order="F")
            cache[key] = (conserve_prim(w, gas.gamma), np.asarray(h, dtype=np.float64),
                          np.asarray(b, dtype=np.float64))
        p, h, b = cache[key]
        ws.append(w); ps_.append(p); hs.append(h); bs.append(b)
    H = np.array(hs)
    # the 1F models carry f alone (held as h); the second distribution is zero
    B = np.zeros_like(H) if KS.nf == 1 else np.array(bs)
    return np.array(ws), np.array(ps_), H, B


def wall_states(KS):
    """KS.ib.bc at every boundary face midpoint (src/Solver/evolve_boundary.jl)."""
    ps, bc = KS.ps, KS.ib.bc
    if KS.dim == 1:
        return [np.asarray(bc(ps.x0), dtype=np.float64)[None, :],
                np.asarray(bc(ps.x1), dtype=np.float64)[None, :]]
    nx, ny = ps.nx, ps.ny
    dx, dy = (ps.x1 - ps.x0) / nx, (ps.y1 - ps.y0) / ny
    xs = [ps.x0 + (i - 0.5) * dx for i in range(1, nx + 1)]
    ys = [ps.y0 + (j - 0.5) * dy for j in range(1, ny + 1)]
    left = [bc(((xs[0] - 0.5 * dx) + (xs[0] - 0.5 * dx)) / 2, ((y - 0.5 * dy) + (y + 0.5 * dy)) / 2) for y in ys]
    right = [bc(((xs[-1] + 0.5 * dx) + (xs[-1] + 0.5 * dx)) / 2, ((y - 0.5 * dy) + (y + 0.5 * dy)) / 2) for y in ys]
    down = [bc(((x - 0.5 * dx) + (x + 0.5 * dx)) / 2, ((ys[0] - 0.5 * dy) + (ys[0] - 0.5 * dy)) / 2) for x in xs]
    up = [bc(((x + 0.5 * dx) + (x - 0.5 * dx)) / 2, ((ys[-1] + 0.5 * dy) + (ys[-1] + 0.5 * dy)) / 2) for x in xs]
    return [np.array(a, dtype=np.float64) for a in (left, right, down, up)]


def init_fvm(KS, precision="fp64"):
    """Device-resident cells and faces for KS.  Returns (ctr, face) in 1D and
    (ctr, a1face, a2face) in 2D, like the reference."""
    vs = KS.vs
    if KS.dim == 1:
        handle = Handle(kb_config(KS, precision), vs.u, None, vs.weights)
    else:
        handle = Handle(kb_config(KS, precision), vs.flat(vs.u), vs.flat(vs.v), vs.flat(vs.weights))
    w, p, h, b = initial_state(KS)
    handle.upload(w, p, h, b)
    for side, prim in enumerate(wall_states(KS)):
        if KS.set.boundary[side] == "maxwell":
            handle.set_wall(side, prim)
    ctr = Cells(KS, handle)
    if KS.dim == 1:
        return ctr, Faces(handle, 0)
    return ctr, Faces(handle, 0), Faces(handle, 1)


def initialize(config, precision=None, **ib_kw):
    """initialize(config) (src/Solver/solver_init.jl:10-48): (KS, ctr, face..., t).

    `config` is a config file path, a dict, or a checkpoint written by
    write_checkpoint (a path ending in ".npz"): like the reference's
    initialize("*.jld2") (src/Solver/solver_init.jl:19-26) the solver set and
    cells come from the file and the time is the checkpoint's.  `precision`
    ("fp64" or "fp32") defaults to "fp64", or to the checkpoint's own.  A
    config with a `mesh` key (a gmsh file) gives the unstructured solve:
    (KS, cells, t) from kitgpu.unstruct.initialize."""
    if isinstance(config, str) and config.endswith(".npz"):
        d = np.load(config, allow_pickle=False)
        meta = json.loads(str(d["set"]))
        KS = solver_set(meta["config"], **meta.get("ib_kw", {}))
        out = init_fvm(KS, precision or meta.get("precision", "fp64"))
        t = read_checkpoint(d, out[0])
        return (KS,) + out + (t,)
    if (isinstance(config, str) and "mesh" in read_dict(config)) or (isinstance(config, dict) and "mesh" in config):
        # a gmsh mesh: the unstructured solve (UnstructPSpace, set_geometry)
        from . import unstruct
        return unstruct.initialize(config, precision or "fp64", **ib_kw)
    KS = solver_set(config, **ib_kw)
    return (KS,) + init_fvm(KS, precision or "fp64") + (0.0,)


def _check_mode(KS, name, given, expect):
    if given is not None and str(given) != str(expect):
        raise ValueError("%s=%r differs from the SolverSet's %r; build a new solver for it"
                         % (name, given, expect))


def timestep(KS, ctr, simTime=0.0):
    """timestep(KS, ctr, simTime) (src/Solver/solver_main.jl:240-342)."""
    return ctr.handle.timestep(KS.set.cfl, simTime, KS.set.maxTime)


def reconstruct(KS, ctr):
    """reconstruct!(KS, ctr)"""
    ctr.handle.reconstruct()


def evolve(KS, ctr, *args, mode=None, bc=None):
    """evolve!(KS, ctr, face, dt) / evolve!(KS, ctr, a1face, a2face, dt)"""
    faces, dt = args[:-1], args[-1]
    _check_mode(KS, "mode", mode, KS.set.flux)
    if bc is not None:
        _check_mode(KS, "bc", bc if isinstance(bc, str) else list(bc),
                    KS.set.boundary[0] if isinstance(bc, str) else KS.set.boundary)
    ctr.handle.evolve(dt)
    for f in faces:
        f.dt = dt


def update(KS, ctr, *args, coll=None, bc=None):
    """update!(KS, ctr, face, dt, residual) / (..., a1face, a2face, dt, residual)"""
    dt, residual = args[-2], args[-1]
    _check_mode(KS, "coll", coll, KS.set.collision)
    r = ctr.handle.update(dt)
    residual[:] = r
    return None


def step(KS, ctr, dt, nsteps=1):
    """nsteps fused reconstruct! -> evolve! -> update! steps; returns the residual."""
    return ctr.handle.step(dt, nsteps)


def solve(KS, ctr, *faces, simTime=0.0, steady=False, chunk=64, adaptive=False):
    """solve! (src/Solver/solver_main.jl:12-150): fixed dt from the initial
    state, nt = floor(maxTime/dt) + 1 iterations, stop when t > maxTime or,
    if steady, when max(res) < 5e-7 (checked every `chunk` steps; chunk=1
    reproduces the per-step test).  adaptive=True is the per-step dt option:
    before every step dt is recomputed from the current state on the device
    (kb_step_cfl) and the run ends at maxTime."""
    t = float(simTime)
    if adaptive:
        res = np.zeros(KS.dim + 2)
        while t < KS.set.maxTime * (1.0 - 1e-14):
            t, res = ctr.handle.step_cfl(KS.set.cfl, t, KS.set.maxTime, chunk)
            if steady and np.max(res) < 5.0e-7:
                break
        return t
    dt = timestep(KS, ctr, t)
    nt = int(math.floor(KS.set.maxTime / dt)) + 1
    it = 0
    res = np.zeros(KS.dim + 2)
    while it < nt:
        n = min(chunk if steady else nt - it, nt - it)
        # the time test of the reference breaks once t > maxTime; with a fixed
        # dt that happens exactly at iteration nt, so the chunk never overshoots
        res = ctr.handle.step(dt, n)
        it += n
        t += n * dt
        if t > KS.set.maxTime:
            break
        if steady and np.max(res) < 5.0e-7:
            break
    for f in faces:
        f.dt = dt
    return t


def extract_sol(KS, ctr):
    """extract_sol (src/IO/io_process.jl:1-40): prim of the physical cells,
    shape (nx, nw) in 1D and (nx, ny, nw) in 2D."""
    s = ctr.handle.download(("prim",))["prim"]
    c = ctr.handle.cfg
    if KS.dim == 1:
        return s[c.ngx:c.ngx + c.nx].copy()
    grid = s.reshape(ctr.handle.nyt, ctr.handle.nxt, -1)
    return grid[c.ngy:c.ngy + c.ny, c.ngx:c.ngx + c.nx].transpose(1, 0, 2).copy()


CKPT_VERSION = 1


def _cell_shape(handle, KS):
    """Per-cell shape of h / b in the checkpoint: (nu,) in 1D and (nv, nu) in
    2D, i.e. a C-order array whose reversed axes are the reference's
    column-major h[u, v] matrix of a ControlVolume2F."""
    return (KS.vs.nu,) if KS.dim == 1 else (KS.vs.nv, KS.vs.nu)


def write_checkpoint(path, KS, ctr, t, slopes=False, precision=None):
    """Checkpoint of the device state (the role of write_jld, src/IO/io_write.jl:34-40,
    which saves Dict("set" => KS, "ctr" => ctr, "t" => t)).

    Keys: "t"; "set" (JSON: the configuration dict the SolverSet was built
    from, its initial-condition keywords, the storage precision); and the
    fields of the reference's ControlVolume2F cells (src/Struct/struct_ctr.jl:94-117)
    as one array per field over all cells incl. ghosts, x fastest (the
    column-major order of the OffsetArray ctr[i, j]): "ctr.w", "ctr.prim"
    [ncell, dim+2], "ctr.h", "ctr.b" [ncell, (nv,) nu], "ctr.sw" [ncell, dim,
    dim+2] (part of the state: ghost cells carry the w slopes bc_extra! copied
    the step before); with slopes=True also "ctr.sh", "ctr.sb"
    [ncell, dim, (nv,) nu] as reconstruct! would store them.  "cells" holds (nx + 2 ngx, ny + 2 ngy)
    and "ghosts" (ngx, ngy): the OffsetArray axes 1-ng : n+ng."""
    hd = ctr.handle
    s = hd.download()
    cs = _cell_shape(hd, KS)
    c = hd.cfg
    prec = precision or ("fp32" if c.precision == N.PRECISION["fp32"] else "fp64")
    meta = dict(version=CKPT_VERSION, config=KS.config, ib_kw=KS.ib_kw or {}, precision=prec)
    arrs = {"t": np.float64(t), "set": np.array(json.dumps(meta)),
            "cells": np.array([hd.nxt, hd.nyt], dtype=np.int64),
            "ghosts": np.array([c.ngx, c.ngy], dtype=np.int64),
            "ctr.w": s["w"], "ctr.prim": s["prim"],
            "ctr.h": s["h"].reshape((hd.ncell,) + cs), "ctr.b": s["b"].reshape((hd.ncell,) + cs)}
    if slopes:
        sw, sh, sb = hd.slopes()
        arrs["ctr.sh"] = sh.reshape((hd.ncell, hd.dim) + cs)
        arrs["ctr.sb"] = sb.reshape((hd.ncell, hd.dim) + cs)
    else:
        sw = np.zeros((hd.ncell, hd.dim, hd.nw))
        N.check(hd.lib.kb_download_slopes(hd.h, N.ptr(sw), None, None))
    # the w slopes are state: ghost cells keep the slopes bc_extra! copied
    # into them the step before, and the face states read them
    arrs["ctr.sw"] = sw
    np.savez(path, **arrs)


def read_checkpoint(path, ctr):
    """Restore the cells of a checkpoint written by write_checkpoint into an
    existing solver of the same shape; returns t.  Raises ValueError when
    the checkpoint's cells or velocity grid do not match the solver's."""
    d = np.load(path, allow_pickle=False) if isinstance(path, str) else path
    hd = ctr.handle
    w, p = d["ctr.w"], d["ctr.prim"]
    h = d["ctr.h"].reshape(len(d["ctr.h"]), -1)
    b = d["ctr.b"].reshape(len(d["ctr.b"]), -1)
    want = (hd.ncell, hd.nw, hd.nvel)
    got = (w.shape[0], w.shape[1], h.shape[1])
    if got != want or p.shape != w.shape or b.shape != h.shape or h.shape[0] != hd.ncell:
        raise ValueError("checkpoint cells (ncell, nw, nvel) = %s do not match the solver's %s"
                         % (got, want))
    hd.upload(w, p, h, b)
    if "ctr.sw" in d:
        hd.upload_slopes(d["ctr.sw"])
    return float(d["t"])
