"""Served stream: continuous batching with HBM-budget admission; each
request's result is the same alone and in the mix (FP32-split; bit-identical
since every request owns its solver), all requests retire, latencies are
reported."""
import numpy as np
import pytest

import kitgpu
from kitgpu import serve as S

pytestmark = pytest.mark.gpu


def test_results_same_alone_and_in_mix(gpu_lib):
    reqs = S.mixed_stream(rate=400.0, duration=0.03, seed=5, max_steps=40, tol=1e-12, scale=0.08)
    assert len(reqs) >= 6
    srv = S.Server(precision="fp32", max_slots=4, chunk=8, hbm_budget=1 << 30)
    m = srv.run(reqs, keep_results=True)
    assert m["requests"] == len(reqs) and m["p50_s"] is not None
    for r in reqs:
        alone = S.Server(precision="fp32", max_slots=1, chunk=40)
        twin = S.Request(r.rid, 0.0, r.config, r.max_steps, r.tol)
        alone.run([twin], keep_results=True)
        assert twin.steps == r.steps
        a, b = r.result["prim"], twin.result["prim"]
        assert np.max(np.abs(a - b) / np.abs(b).clip(1e-30)) < 1e-12


def test_admission_respects_budget(gpu_lib):
    reqs = S.mixed_stream(rate=400.0, duration=0.03, seed=9, max_steps=10, tol=1e-12, scale=0.08)
    budget = 2 * max(S.estimate_bytes(r.config, "fp32") for r in reqs)
    peak = []
    srv = S.Server(precision="fp32", max_slots=16, chunk=5, hbm_budget=budget)

    def on_retire(r):
        peak.append(r.bytes)

    m = srv.run(reqs, on_retire=on_retire)
    assert m["requests"] == len(reqs)
    assert all(r.finished >= r.admitted >= r.arrival - 1e-9 for r in srv.done)
