"""The project autotuner (kitgpu.tune) on the CPU, with fake handles whose
simulated stage times depend on the launch shape: each search picks the
fastest candidate (the update shape first, then the moment pass given it),
skips shapes the library refuses, writes its choice to the cache under the
problem's signature, and a later call with the same signature takes the
cached shape without stepping."""
import json
import time
import types

import numpy as np
import pytest

from kitgpu import tune
from kitgpu import _native as N
from kitgpu._native import KitGPUError


@pytest.fixture
def cache(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setattr(tune, "CACHE", str(path))
    return path


class FakeHandle:
    """Simulated per-step stage times (ms): the update pass by (tx, bs, ry),
    the moment pass by faces per warp."""

    def __init__(self, dim=2, nx=512, ny=512, nvel=4096, flux=2, coll=0, prec=1,
                 upd_best=(4, 64, 64), mom_best=2):
        self.cfg = types.SimpleNamespace(dim=dim, nx=nx, ny=ny, flux=flux, collision=coll,
                                         precision=prec)
        self.dim, self.nvel = dim, nvel
        self.upd_best, self.mom_best = upd_best, mom_best
        self.shape = None
        self.steps = 0
        self.timed = None

    def set_tuning(self, march_tx=0, march_ry=0, march_bs=0, mom_ts=0):
        self.shape = (march_tx, march_bs, march_ry, mom_ts)

    def set_timing(self, on=True):
        self.timed = [0.0, 0, 0.0, 0] if on else None

    def step(self, dt, n):
        self.steps += n
        if self.timed is not None:
            tx, bs, ry, ts = self.shape
            upd = 6.0 + (0.0 if (tx, bs, ry) == self.upd_best else 0.1 * (1 + tx + bs / 64 + ry / 16))
            mom = 5.0 + (0.0 if ts == self.mom_best else 0.05 * ts)
            self.timed = [self.timed[0] + n * upd, self.timed[1] + n,
                          self.timed[2] + n * mom, self.timed[3] + n]

    def timing(self):
        u, nu, m, nm = self.timed
        return {"update": (u, nu), "moments": (m, nm)}


@pytest.mark.parametrize("upd_best,mom_best", [((4, 64, 64), 2), ((2, 128, 16), 8), ((2, 64, 32), 4)])
def test_autotune_picks_fastest_and_caches(cache, upd_best, mom_best):
    hd = FakeHandle(upd_best=upd_best, mom_best=mom_best)
    best, timings = tune.autotune(hd, 1e-3, steps=2)
    assert best == dict(march_tx=upd_best[0], march_bs=upd_best[1], march_ry=upd_best[2], mom_ts=mom_best)
    assert hd.shape == (upd_best[0], upd_best[1], upd_best[2], mom_best)  # left set on the handle
    n_cand = len(tune.MARCH_TX) * len(tune.MARCH_BS) * len(tune.MARCH_RY)
    assert len(timings["march"]) == n_cand and len(timings["moments"]) == len(tune.MOM_TS)
    stored = json.load(open(cache))
    assert stored == {tune.signature(hd): best}
    # same signature: the cached shape, no search
    hd2 = FakeHandle(upd_best=(2, 64, 16), mom_best=4)
    best2, t2 = tune.autotune(hd2, 1e-3)
    assert best2 == best and t2 is None and hd2.steps == 0
    assert hd2.shape == (best["march_tx"], best["march_bs"], best["march_ry"], best["mom_ts"])


def test_autotune_1d_has_one_row_option(cache):
    hd = FakeHandle(dim=1, nx=200, ny=1, nvel=101, flux=0, coll=1, upd_best=(2, 128, 1), mom_best=4)
    best, timings = tune.autotune(hd, 1e-3)
    assert best["march_ry"] == 1 and best["march_tx"] == 2 and best["march_bs"] == 128
    assert len(timings["march"]) == len(tune.MARCH_TX) * len(tune.MARCH_BS)


def test_signature_separates_problem_classes():
    a = FakeHandle()
    sig = tune.signature(a)
    assert sig != tune.signature(FakeHandle(nx=32, ny=32))      # size class
    assert sig != tune.signature(FakeHandle(nvel=784))          # velocity count
    assert sig != tune.signature(FakeHandle(prec=0))            # precision
    assert sig != tune.signature(FakeHandle(coll=1))            # collision model
    assert sig == tune.signature(FakeHandle(nx=500, ny=520))    # same class


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t


def test_autotune_unstruct_skips_refused_shapes(cache, monkeypatch):
    clock = FakeClock()
    monkeypatch.setattr(time, "perf_counter", clock)
    cost = {4: 0.9, 8: 0.7, 12: 0.6, 16: 0.65, 24: 0.8}  # 32 refused (shared memory)

    class US:
        nvel, ncell = 256, 294912
        cfg = types.SimpleNamespace(collision=0, precision=1)

        def __init__(self):
            self.cb = None

        def set_tuning(self, cb):
            if cb not in cost:
                raise KitGPUError(N.KB_ERR_CONFIG, "more shared memory than a CTA may have")
            self.cb = cb

        def step(self, dt, n):
            clock.t += n * cost[self.cb] * 1e-3

    hd = US()
    best, tim = tune.autotune_unstruct(hd, 1e-3, steps=10)
    assert best == 12 and hd.cb == 12
    assert set(tim) == {"cb%d" % k for k in cost}
    assert tim["cb12"] == pytest.approx(0.6)
    assert json.load(open(cache)) == {tune.unstruct_signature(hd): {"cells_per_cta": 12}}


def test_autotune_batch_fp32_only_and_cached(cache, monkeypatch):
    clock = FakeClock()
    monkeypatch.setattr(time, "perf_counter", clock)
    fastest = (16, 128, 1)

    class Batch:
        prec = "fp32"
        n = 512
        nu = np.array([48, 200, 96])
        KS = [types.SimpleNamespace(set=types.SimpleNamespace(collision="shakhov"))]

        def __init__(self):
            self.shape = None
            self.steps = 0

        def cell_velocity_points(self):
            return 14_143_356

        def set_tuning(self, seg, threads, persist):
            self.shape = (seg, threads, persist)

        def step(self, n):
            self.steps += n
            clock.t += n * (0.196 if self.shape == fastest else 0.25) * 1e-3

    b = Batch()
    best, tim = tune.autotune_batch(b, steps=50)
    assert best == dict(seg=16, threads=128, persist=1) and b.shape == fastest
    assert len(tim) == len(tune.BATCH_SHAPES) * len(tune.BATCH_PERSIST)
    b2 = Batch()
    assert tune.autotune_batch(b2) == (best, None) and b2.steps == 0
    b64 = Batch()
    b64.prec = "fp64"
    assert tune.autotune_batch(b64) == (None, None) and b64.steps == 0
