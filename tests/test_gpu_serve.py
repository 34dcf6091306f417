"""Served stream: continuous batching with HBM-budget admission.  In the mix
the 1D requests share the pool's fused launches and the 2D requests the
group's launches (one launch per step kernel for all resident 2D solves);
each request's result is bit-identical alone and in the mix, all requests
retire, latencies are reported."""
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


def test_pooled_1d_requests_share_launches(gpu_lib):
    """The 1D requests of a stream are advanced together by the pool's fused
    launches: far fewer pool launches than pooled request-steps."""
    reqs = S.mixed_stream(rate=400.0, duration=0.05, seed=11, max_steps=40, tol=1e-12, scale=0.08)
    n1d = sum(1 for r in reqs if r.config["space"] == "1d2f1v")
    assert n1d >= 3
    srv = S.Server(precision="fp32", max_slots=8, chunk=8, hbm_budget=1 << 30)
    m = srv.run(reqs)
    assert m["requests"] == len(reqs)
    assert 0 < m["pool_launches"] < n1d * 40 * 2


def test_2d_requests_share_group_launches(gpu_lib):
    """The 2D requests of a stream are advanced together by the group's
    launches: far fewer group launches than 2D request-steps times the
    kernels of a step."""
    reqs = S.mixed_stream(rate=400.0, duration=0.05, seed=11, max_steps=40, tol=1e-12, scale=0.08)
    n2d = sum(1 for r in reqs if r.config["space"] == "2d2f2v")
    assert n2d >= 2
    srv = S.Server(precision="fp32", max_slots=8, chunk=8, hbm_budget=1 << 30)
    m = srv.run(reqs)
    assert m["requests"] == len(reqs)
    assert 0 < m["group_launches"] < n2d * 40 * 8


def test_pool_join_leave_and_accuracy(gpu_lib):
    """Solves join a pool while others run and leave it: each result equals
    the same solve alone in a pool bit for bit, stays within 1e-5 of the
    plain FP64 single solve (rho, U, T), and freed slots are reused."""
    from kitgpu import batch as KB
    from cases import rho_u_t_error, sod
    cfgs = [sod(nx=60, nu=40), sod(nx=37, nu=33), sod(nx=90, nu=64), sod(nx=16, nu=7)]
    sets = [kitgpu.solver_set(c) for c in cfgs]

    def alone(KS, n):
        p = KB.Pool(KS, max_instances=1, max_cells=256)
        slot, dt = p.add(KS)
        p.step(n)
        out = p.download(slot)
        p.close()
        return out, dt

    pool = KB.Pool(sets[0], max_instances=3, max_cells=256)
    s0, dt0 = pool.add(sets[0])
    pool.step(10)
    s1, dt1 = pool.add(sets[1])      # joins a running pool
    pool.step(10)
    a0 = pool.download(s0)
    pool.remove(s0)                  # leaves; its ranges are reused below
    s2, dt2 = pool.add(sets[2])
    s3, dt3 = pool.add(sets[3])
    pool.step(20)
    a1, a2, a3 = pool.download(s1), pool.download(s2), pool.download(s3)
    for (got, KS, n, dt) in ((a0, sets[0], 20, dt0), (a1, sets[1], 30, dt1), (a2, sets[2], 20, dt2),
                             (a3, sets[3], 20, dt3)):
        ref, dtr = alone(KS, n)
        assert dtr == dt
        for k in ("w", "prim", "h", "b"):
            assert np.array_equal(got[k], ref[k]), k
        ctr, face = kitgpu.init_fvm(KS, "fp64")
        assert kitgpu.timestep(KS, ctr, 0.0) == pytest.approx(dt, rel=1e-14)
        ctr.handle.step(dt, n)
        single = ctr.handle.download()
        assert max(rho_u_t_error(got["prim"], single["prim"])) < 1e-5
    pool.close()
