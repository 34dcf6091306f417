"""The served stream's scheduler (kitgpu.serve.Server) on the CPU, with fake
device objects in place of the C ABI's handles, 1D pool and 2D group: every
request retires at its tolerance or at its step cap, admission keeps to the
slot count and the HBM budget, and requests are routed to the pool (1D
FP32), the group (small 2D FP32 KCU cavities) or a stream of their own.
The fakes advance a per-request residual 0.3^steps or 0.97^steps (the
latter never reaches the tolerance, so those requests stop at the cap)."""

import numpy as np
import pytest

from kitgpu import serve as S
from kitgpu import _native as N
from kitgpu._native import KitGPUError


class Fleet:
    """What is resident on the fake device, with peaks."""

    def __init__(self):
        self.handles = {}      # id -> bytes estimate of live handles
        self.pool_slots = 0
        self.peak_residents = 0
        self.peak_bytes = 0
        self.routes = {}       # (nx, ny, nu) -> "stream" | "pool" | "group"

    def note(self):
        self.peak_residents = max(self.peak_residents, len(self.handles) + self.pool_slots)
        self.peak_bytes = max(self.peak_bytes, sum(self.handles.values()))


def decay_of(nx):
    return 0.3 if nx % 2 == 0 else 0.97


def make_fakes(fleet, precision):
    class FakeHandle:
        def __init__(self, cfg, u, v, w):
            self.cfg = cfg
            self.dim = cfg.dim
            self.nvel = len(u)
            self.steps = 0
            self.pending = 0
            self.decay = decay_of(cfg.nx)
            self.key = (cfg.nx, cfg.ny, cfg.nu)
            fleet.routes[self.key] = "stream"
            ny = cfg.ny if cfg.dim == 2 else 1
            fake_cfg = dict(space="%dd2f%dv" % (cfg.dim, cfg.dim), nx=cfg.nx, ny=ny,
                            nu=cfg.nu, nv=cfg.nv)
            fleet.handles[id(self)] = S.estimate_bytes(fake_cfg, precision)
            fleet.note()

        def set_tuning(self, **kw):
            pass

        def init_equilibrium(self, w, p):
            pass

        def set_wall(self, side, prim):
            pass

        def timestep(self, cfl, t, tmax):
            return 1e-3

        def step_async(self, dt, n):
            assert self.pending == 0, "a chunk was enqueued on a busy handle"
            self.pending = n

        def query(self):
            self.steps += self.pending
            self.pending = 0
            return True, np.full(self.dim + 2, self.decay ** self.steps)

        def download(self, want=("w", "prim", "h", "b")):
            return {k: np.zeros(1) for k in want}

        def close(self):
            del fleet.handles[id(self)]

    class FakePool:
        def __init__(self, KS, max_instances=64, max_cells=1 << 17):
            self.key = S.KBATCH.pool_key(KS)
            self.cap, self.max_cells = max_instances, max_cells
            self.slots = {}  # slot -> [steps, decay, cells]
            self.nlaunch = 0

        def add(self, KS):
            cells = KS.ps.nx + 2 * KS.ps.ng
            if (len(self.slots) >= self.cap
                    or sum(s[2] for s in self.slots.values()) + cells > self.max_cells):
                raise KitGPUError(N.KB_ERR_NOMEM, "pool full")
            slot = min(set(range(self.cap)) - set(self.slots))
            self.slots[slot] = [0, decay_of(KS.ps.nx), cells]
            fleet.routes[(KS.ps.nx, 1, KS.vs.nu)] = "pool"
            fleet.pool_slots += 1
            fleet.note()
            return slot, 1e-3

        def step(self, n, tol):
            res = np.zeros((self.cap, 3))
            for k, s in self.slots.items():
                s[0] += n
                res[k] = s[1] ** s[0]
            self.nlaunch += n
            return res

        def launches(self):
            return self.nlaunch

        def download(self, slot, want=("w", "prim", "h", "b")):
            return {k: np.zeros(1) for k in want}

        def remove(self, slot):
            del self.slots[slot]
            fleet.pool_slots -= 1

        def close(self):
            pass

    class FakeGroup:
        def __init__(self, capacity=64):
            self.members = []
            self.nlaunch = 0

        def add(self, handle, dt):
            if handle.cfg.nx > 40:  # the ABI refuses grids its cell blocks do not cover
                raise KitGPUError(N.KB_ERR_CONFIG, "grid too large for the group")
            self.members.append(handle)
            fleet.routes[handle.key] = "group"

        def remove(self, handle):
            self.members.remove(handle)

        def step_async(self, n):
            for h in self.members:
                h.steps += n
            self.nlaunch += 8 * n

        def query(self):
            res = np.array([np.full(4, h.decay ** h.steps) for h in self.members]).reshape(-1, 4)
            return True, res, np.zeros(len(self.members), dtype=np.int32)

        def launches(self):
            return self.nlaunch

        def close(self):
            pass

    return FakeHandle, FakePool, FakeGroup


@pytest.fixture
def fake_device(monkeypatch):
    def install(precision):
        fleet = Fleet()
        H, P, G = make_fakes(fleet, precision)
        monkeypatch.setattr(S, "Handle", H)
        monkeypatch.setattr(S.KBATCH, "Pool", P)
        monkeypatch.setattr(S.KGROUP, "Group", G)
        return fleet
    return install


def stream(seed, n_min=12):
    reqs = S.mixed_stream(rate=2000.0, duration=0.02, seed=seed, max_steps=40, tol=1e-6, scale=0.08)
    assert len(reqs) >= n_min
    return reqs


def check_retired(srv, reqs, chunk):
    assert sorted(r.rid for r in srv.done) == sorted(r.rid for r in reqs)
    for r in srv.done:
        assert r.finished >= r.admitted >= r.arrival - 1e-9
        assert r.steps % chunk == 0 and r.steps <= r.max_steps
        converged = float(np.max(r.residual)) < r.tol
        assert converged or r.steps == r.max_steps
        if decay_of(r.config["nx"]) == 0.3:  # converges after 12 steps: first whole chunk past it
            assert r.steps == 16
        else:
            assert not converged


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_every_request_retires_fp32(fake_device, seed):
    fleet = fake_device("fp32")
    reqs = stream(seed)
    srv = S.Server(precision="fp32", max_slots=6, chunk=8, hbm_budget=1 << 30)
    m = srv.run(reqs, keep_results=True)
    assert m["requests"] == len(reqs)
    check_retired(srv, reqs, 8)
    assert all(r.result is not None for r in srv.done)
    assert fleet.peak_residents <= 6
    assert not fleet.handles and fleet.pool_slots == 0  # everything released


def test_routing(fake_device):
    fleet = fake_device("fp32")
    reqs = stream(4)
    # a group threshold inside the stream's 2D sizes, so both 2D routes occur
    srv = S.Server(precision="fp32", max_slots=8, chunk=8, hbm_budget=1 << 30, group_max_cv=60000)
    m = srv.run(reqs)
    assert set(fleet.routes.values()) == {"pool", "group", "stream"}
    for r in reqs:
        c = r.config
        if c["space"] == "1d2f1v":
            key, want = (c["nx"], 1, c["nu"]), "pool"
        else:
            key = (c["nx"], c["ny"], c["nu"])
            small = c["nx"] * c["ny"] * c["nu"] * c["nv"] <= srv.group_max_cv and c["nx"] <= 40
            want = "group" if small else "stream"
        assert fleet.routes[key] == want, (key, want)
    assert m["pool_launches"] > 0 and m["group_launches"] > 0


def test_fp64_requests_use_their_own_streams(fake_device):
    fleet = fake_device("fp64")
    reqs = stream(5)
    srv = S.Server(precision="fp64", max_slots=4, chunk=8, hbm_budget=1 << 30)
    m = srv.run(reqs)
    assert m["requests"] == len(reqs)
    check_retired(srv, reqs, 8)
    assert set(fleet.routes.values()) == {"stream"}
    assert m["pool_launches"] == 0 and m["group_launches"] == 0
    assert fleet.peak_residents <= 4


def test_admission_keeps_to_the_hbm_budget(fake_device):
    """With a budget of two of the largest requests, the handles resident at
    once never hold more than the budget."""
    fleet = fake_device("fp64")
    reqs = stream(6)
    budget = 2 * max(S.estimate_bytes(r.config, "fp64") for r in reqs)
    srv = S.Server(precision="fp64", max_slots=16, chunk=8, hbm_budget=budget)
    m = srv.run(reqs)
    assert m["requests"] == len(reqs)
    assert fleet.peak_bytes <= budget


def test_a_request_larger_than_the_budget_runs_alone(fake_device):
    fleet = fake_device("fp64")
    reqs = stream(7)
    small = min(S.estimate_bytes(r.config, "fp64") for r in reqs)
    srv = S.Server(precision="fp64", max_slots=16, chunk=8, hbm_budget=small)
    m = srv.run(reqs)
    assert m["requests"] == len(reqs)
    assert fleet.peak_residents == 1  # admitted only when nothing else is resident


def test_group_refusal_falls_back_to_own_stream(fake_device):
    """A 2D request under the group's size threshold that the group kernels
    do not cover (the ABI refuses it) runs on its own stream instead."""
    fleet = fake_device("fp32")
    reqs = [S.Request(0, 0.0, S.cavity_request(48, 8, 1e-2), 40, 1e-6),   # refused: own stream
            S.Request(1, 0.0, S.cavity_request(12, 8, 1e-2), 40, 1e-6),   # grouped
            S.Request(2, 0.0, S.sod_request(64, 32), 40, 1e-6)]           # pooled
    srv = S.Server(precision="fp32", max_slots=4, chunk=8, hbm_budget=1 << 30)
    m = srv.run(reqs)
    assert m["requests"] == 3
    assert fleet.routes[(48, 48, 8)] == "stream"
    assert fleet.routes[(12, 12, 8)] == "group"
    assert fleet.routes[(64, 1, 32)] == "pool"
    check_retired(srv, reqs, 8)
