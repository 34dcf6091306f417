"""Continuous-batching service for a stream of DVM solves.

Requests arrive over time (Poisson).  1D requests that the batch kernel
covers (1D2F1V, KFVS, fixed boundaries) join a resident pool (batch.Pool,
kb_pool_*): one fused launch per step advances every resident 1D request,
requests join and leave between chunks of steps, and a request's result does
not depend on who else shares the launch.  The small 2D cavities join a
group (group.Group, kb_group_*): one launch of each step kernel advances
every grouped request, requests join and leave between the group's chunks,
and each result is bit-identical to the same solve in a group of its own.
Every other request owns a libkitgpu handle with its own CUDA stream, so its
steps run concurrently with the pool, the group and each other.  The loop admits queued
requests whenever a slot and the HBM budget allow, advances the pool by a
chunk on a worker thread (so the loop keeps feeding the 2D solves while the
pool steps), enqueues a chunk for every idle handle (kb_step_async), polls
completions (kb_query) and retires a request when its residual (reference
definition, src/Solver/solver_update.jl:86-88) falls below the tolerance or
it reaches its step limit; its final state is downloaded and its memory
returned to the budget before the next admission.  A request's step limit
should be a multiple of the chunk: steps are counted in whole chunks.

The mixed stream: 60 % 1D Sod tubes (cells log-uniform in [64, 2048],
velocities in [32, 256]) and 40 % 2D lid-driven cavities (cells log-uniform
in [16^2, 128^2], velocity grids in [16^2, 48^2], Kn log-uniform in
[1e-4, 1]).
"""
import concurrent.futures
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import batch as KBATCH
from . import group as KGROUP
from ._native import KitGPUError
from .setup import solver_set
from .solver import Handle, initial_cells, kb_config, wall_states


def sod_request(nx, nu, Kn=1e-3):
    return dict(matter="gas", case="sod", space="1d2f1v", flux="kfvs", collision="shakhov",
                nSpecies=1, interpOrder=2, limiter="vanleer", boundary="fix", cfl=0.5,
                maxTime=1e9, x0=0.0, x1=1.0, nx=int(nx), nxg=0, umin=-5.0, umax=5.0,
                nu=int(nu), vMeshType="newton", knudsen=Kn, mach=0.0, prandtl=2.0 / 3.0,
                inK=2.0, omega=0.81, alphaRef=1.0, omegaRef=0.5)


def cavity_request(n, nv, Kn):
    return dict(matter="gas", case="cavity", space="2d2f2v", flux="kcu", collision="shakhov",
                nSpecies=1, interpOrder=2, limiter="vanleer", boundary="maxwell", cfl=0.8,
                maxTime=1e9, x0=0.0, x1=1.0, nx=int(n), nxg=0, y0=0.0, y1=1.0, ny=int(n), nyg=0,
                umin=-5.0, umax=5.0, nu=int(nv), vmin=-5.0, vmax=5.0, nv=int(nv),
                vMeshType="newton", knudsen=float(Kn), mach=0.0, prandtl=2.0 / 3.0, inK=1.0,
                omega=0.72, alphaRef=1.0, omegaRef=0.5, uLid=0.15, vLid=0.0, tLid=1.0)


@dataclass
class Request:
    rid: int
    arrival: float
    config: dict
    max_steps: int
    tol: float
    # filled by the server
    admitted: float = None
    finished: float = None
    steps: int = 0
    residual: np.ndarray = None
    result: dict = None
    cv_per_step: int = 0
    bytes: int = 0

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival


def mixed_stream(rate, duration, seed=20261203, max_steps=200, tol=1e-6, frac_1d=0.6,
                 scale=1.0):
    """Poisson arrivals at `rate` per second over `duration` seconds.  `scale`
    shrinks the size ranges (tests use small requests)."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        if rng.uniform() < frac_1d:
            nx = int(round(math.exp(rng.uniform(math.log(64), math.log(2048))) * scale))
            nu = int(rng.integers(32, 257) * min(1.0, scale * 4))
            cfg = sod_request(max(nx, 8), max(nu, 16))
        else:
            n = int(round(math.exp(rng.uniform(math.log(16), math.log(128))) * scale))
            nv = int(rng.integers(16, 49))
            Kn = math.exp(rng.uniform(math.log(1e-4), math.log(1.0)))
            cfg = cavity_request(max(n, 4), nv, Kn)
        out.append(Request(len(out), t, cfg, max_steps, tol))
    return out


# Launch shapes of the served 2D solves.  Served grids are small (16^2 to
# 128^2 cells): the shapes that suit one large solve give them few CTAs, each
# a long serial march.  Two-column strips of 8 rows with one velocity per
# thread in the update pass and two faces per warp in the moment pass were
# the fastest on every served size measured (16^2 x 21^2 to 128^2 x 48^2 cells
# x velocities: 1.3-2x the default shapes).  Fixed rather than autotuned per
# request: a tuning search would advance the request's own solution.
SERVE_SHAPE_2D = dict(march_tx=2, march_ry=8, march_bs=128, mom_ts=2)


def estimate_bytes(cfg, precision):
    """Device bytes of a handle for `cfg` (distributions x2 buffers dominate)."""
    d = int(cfg["space"][0])
    ncell = (cfg["nx"] + 2 * cfg.get("nxg", 0)) * ((cfg["ny"] + 2 * cfg.get("nyg", 0)) if d == 2 else 1)
    nvel = cfg["nu"] * (cfg["nv"] if d == 2 else 1)
    esz = 4 if precision == "fp32" else 8
    nface = (cfg["nx"] + 1) * (cfg.get("ny", 1) if d == 2 else 1) * (2 if d == 2 else 1)
    return 4 * ncell * ((nvel + 3) // 4 * 4) * esz + ncell * 1024 + nface * 512 + (1 << 20)


def pool_bytes(max_cells, max_nu=256):
    """Device bytes of a 1D pool: FP32 h, b (two buffers each) and the FP64
    staging array over max_cells x max_nu values, plus per-cell state."""
    return max_cells * max_nu * (4 * 4 + 8) + max_cells * 512 + (8 << 20)


@dataclass
class Server:
    precision: str = "fp32"
    hbm_budget: int = 64 << 30
    max_slots: int = 64
    chunk: int = 20
    pool_1d: bool = True          # 1D requests share one fused launch (FP32 only)
    pool_cells: int = None        # cell capacity of the pool; None: from the HBM budget
    shape_2d: dict = field(default_factory=lambda: dict(SERVE_SHAPE_2D))  # None: library defaults
    group_2d: bool = True         # small 2D requests share launches (kb_group_*)
    # 2D requests of at most this many cell-velocity points per step join the
    # group; larger ones keep their own stream.  Measured on 24 cavities of the
    # mix: all in one group 3.5e10 cv/s (each launch waits for its largest
    # member), each on its own stream 4.0e10, the 12 smallest grouped and the
    # rest on streams 4.1e10 -- the small requests' latency-bound steps share
    # launches, the large ones run unhindered.
    group_max_cv: int = 1 << 21
    done: list = field(default_factory=list)

    def run(self, requests, time_scale=1.0, keep_results=False, on_retire=None):
        """Serve `requests` (sorted by arrival).  Arrival times are honoured in
        wall time divided by time_scale.  Returns summary metrics."""
        pending = sorted(requests, key=lambda r: r.arrival)
        if self.pool_cells is None:  # a quarter of the budget, at most 64 slots of 2048 cells
            self.pool_cells = int(min(self.max_slots * 2052,
                                      max(4096, self.hbm_budget // 4 // (256 * 24))))
        queue, active, pooled = [], [], []
        grouped, joining = [], []  # 2D requests in the group / admitted, joining at its next chunk
        group = None
        group_job = None  # steps of the group chunk in flight
        self.group_launches = 0
        used = 0
        pool = None
        pool_job = None  # (future, steps, launches before) of the pool chunk in flight
        worker = concurrent.futures.ThreadPoolExecutor(max_workers=1)
        self.pool_launches = 0
        t0 = time.perf_counter()
        cv_total = 0
        i = 0

        def retire(r, state):
            nonlocal used
            r.finished = (time.perf_counter() - t0) * time_scale
            if keep_results:
                r.result = state
            self.done.append(r)
            if on_retire:
                on_retire(r)

        while (i < len(pending) or queue or active or pooled or pool_job is not None or grouped
               or joining):
            now = (time.perf_counter() - t0) * time_scale
            while i < len(pending) and pending[i].arrival <= now:
                queue.append(pending[i])
                i += 1
            # admission: FIFO while a slot and the HBM budget allow
            while queue and len(active) + len(pooled) + len(grouped) + len(joining) < self.max_slots:
                r = queue[0]
                KS = solver_set(r.config)
                use_pool = (self.pool_1d and self.precision == "fp32" and KBATCH.poolable(KS)
                            and (pool is None or KBATCH.pool_key(KS) == pool.key)
                            and KS.ps.nx + 2 * KS.ps.ng <= self.pool_cells)
                if use_pool and pool_job is not None:
                    break  # the pool's chunk is in flight: join it when it returns
                if use_pool and pool is None:
                    need = pool_bytes(self.pool_cells)
                    if used + need > self.hbm_budget and (active or pooled or grouped or joining):
                        break
                    pool = KBATCH.Pool(KS, max_instances=self.max_slots, max_cells=self.pool_cells)
                    used += need
                if use_pool:
                    try:
                        r.slot, r.dt = pool.add(KS)
                    except Exception:
                        if not pooled:
                            raise
                        break  # pool capacity used up: wait for a retirement
                    queue.pop(0)
                    r.handle = None
                    r.bytes = 0
                    r.cv_per_step = KS.ps.nx * KS.vs.nu
                    r.admitted = (time.perf_counter() - t0) * time_scale
                    pooled.append(r)
                    continue
                need = estimate_bytes(r.config, self.precision)
                if used + need > self.hbm_budget and (active or pooled or grouped or joining):
                    break
                queue.pop(0)
                vs = KS.vs
                if KS.dim == 1:
                    h = Handle(kb_config(KS, self.precision), vs.u, None, vs.weights)
                else:
                    h = Handle(kb_config(KS, self.precision), vs.flat(vs.u), vs.flat(vs.v),
                               vs.flat(vs.weights))
                if KS.dim == 2 and self.precision == "fp32" and self.shape_2d:
                    h.set_tuning(**self.shape_2d)
                # the Sod and cavity presets start in equilibrium: only w and
                # prim cross the bus, h and b are built on the device
                w, p = initial_cells(KS)
                h.init_equilibrium(w, p)
                for side, prim in enumerate(wall_states(KS)):
                    if KS.set.boundary[side] == "maxwell":
                        h.set_wall(side, prim)
                r.dt = h.timestep(KS.set.cfl, 0.0, KS.set.maxTime)
                r.handle = h
                r.bytes = need
                r.cv_per_step = h.cfg.nx * (h.cfg.ny if h.dim == 2 else 1) * h.nvel
                r.admitted = (time.perf_counter() - t0) * time_scale
                used += need
                r.inflight = 0
                if self.group_2d and KGROUP.groupable(h) and r.cv_per_step <= self.group_max_cv:
                    joining.append(r)
                else:
                    active.append(r)
            # enqueue a chunk for every idle resident handle
            for r in active:
                if r.inflight == 0:
                    n = min(self.chunk, r.max_steps - r.steps)
                    r.handle.step_async(r.dt, n)
                    r.inflight = n
            # one chunk of the pool (every resident 1D request in each launch)
            # runs on a worker thread, so that this loop keeps feeding and
            # polling the 2D solves meanwhile; joins and leaves of the pool
            # happen only between its chunks
            if pooled and pool_job is None:
                l0 = pool.launches()
                pool_job = (worker.submit(pool.step, self.chunk, min(r.tol for r in pooled)),
                            self.chunk, l0)
            if pool_job is not None and pool_job[0].done():
                fut, n, l0 = pool_job
                pool_job = None
                res = fut.result()
                self.pool_launches += pool.launches() - l0
                still = []
                for r in pooled:
                    r.steps += n
                    cv_total += n * r.cv_per_step
                    r.residual = res[r.slot].copy()
                    if r.steps >= r.max_steps or float(np.max(r.residual)) < r.tol:
                        state = pool.download(r.slot, ("w", "prim")) if keep_results else None
                        pool.remove(r.slot)
                        retire(r, state)
                    else:
                        still.append(r)
                pooled = still
            # the group of 2D solves: one launch per step kernel for all of
            # them; requests join and leave between its chunks
            if group_job is None and (grouped or joining):
                if group is None:
                    group = KGROUP.Group(self.max_slots)
                for r in joining:
                    try:
                        group.add(r.handle, r.dt)
                        grouped.append(r)
                    except KitGPUError:  # not covered by the group kernels: its own stream
                        active.append(r)
                joining = []
                if grouped:
                    l0 = group.launches()
                    group.step_async(self.chunk)
                    group_job = (self.chunk, l0)
            elif group_job is not None:
                ready, gres, _ = group.query()
                if ready:
                    n, l0 = group_job
                    group_job = None
                    self.group_launches += group.launches() - l0
                    by_handle = {id(r.handle): r for r in grouped}
                    still = []
                    for k, hd in enumerate(list(group.members)):
                        r = by_handle[id(hd)]
                        r.steps += n
                        cv_total += n * r.cv_per_step
                        r.residual = gres[k].copy()
                        if r.steps >= r.max_steps or float(np.max(r.residual)) < r.tol:
                            group.remove(hd)
                            state = hd.download(("w", "prim")) if keep_results else None
                            hd.close()
                            r.handle = None
                            used -= r.bytes
                            retire(r, state)
                        else:
                            still.append(r)
                    grouped = still
            # poll completions of the handles
            still = []
            for r in active:
                ready, res = r.handle.query()
                if not ready:
                    still.append(r)
                    continue
                r.steps += r.inflight
                cv_total += r.inflight * r.cv_per_step
                r.inflight = 0
                r.residual = res
                if r.steps >= r.max_steps or float(np.max(res)) < r.tol:
                    state = r.handle.download(("w", "prim")) if keep_results else None
                    r.handle.close()
                    r.handle = None
                    used -= r.bytes
                    retire(r, state)
                else:
                    still.append(r)
            active = still
            if (not active and not pooled and not queue and not grouped and not joining
                    and i < len(pending)):
                # idle until the next arrival
                wait = (pending[i].arrival - now) / time_scale
                if wait > 0:
                    time.sleep(min(wait, 0.01))
        wall = time.perf_counter() - t0
        worker.shutdown(wait=True)
        if group is not None:
            group.close()
        if pool is not None:
            pool.close()
        lat = np.array([r.latency for r in self.done if r.latency is not None]) / time_scale
        return dict(requests=len(self.done), wall_s=wall, cv_updates=cv_total,
                    throughput=cv_total / wall if wall > 0 else 0.0,
                    p50_s=float(np.percentile(lat, 50)) if len(lat) else None,
                    p99_s=float(np.percentile(lat, 99)) if len(lat) else None,
                    precision=self.precision, max_slots=self.max_slots,
                    hbm_budget=self.hbm_budget, pool_launches=self.pool_launches,
                    group_launches=self.group_launches)
