"""Batched ensemble (one persistent launch per step over a ragged index):
every instance equals its own single solve, in FP64 to 1e-12 and in the
FP32-split form to 1e-5; an instance's result does not depend on the rest of
the batch; converged instances stop."""
import numpy as np
import pytest

import kitgpu
from kitgpu import batch as KB
from cases import rho_u_t_error

pytestmark = pytest.mark.gpu


def small_ensemble(n=6, seed=7, coll="shakhov"):
    rng = np.random.default_rng(seed)
    cfgs = []
    for _ in range(n):
        cfgs.append(KB.shock_config(rng.uniform(1.2, 8.0), int(rng.integers(20, 90)),
                                    int(rng.integers(48, 201)), coll=coll))
    return cfgs


def single(KS, dt, nsteps, precision="fp64"):
    ctr, face = kitgpu.init_fvm(KS, precision)
    ctr.handle.step(dt, nsteps)
    return ctr.handle.download()


@pytest.mark.parametrize("coll", ["shakhov", "bgk"])
def test_batch_fp64_equals_single_solves(gpu_lib, coll):
    sets = KB.solver_sets(small_ensemble(coll=coll))
    bt = KB.Batch(sets, "fp64")
    bt.upload_initial()
    dt = bt.timestep()
    for k, KS in enumerate(sets):
        ctr, face = kitgpu.init_fvm(KS)
        assert dt[k] == pytest.approx(kitgpu.timestep(KS, ctr, 0.0), rel=1e-14)
    bt.step(30)
    outs = bt.download()
    for k, KS in enumerate(sets):
        ref = single(KS, dt[k], 30)
        e = rho_u_t_error(outs[k]["prim"], ref["prim"])
        assert max(e) < 1e-12, (k, e)
        assert np.max(np.abs(outs[k]["h"] - ref["h"])) < 1e-12 * np.max(ref["h"])


def test_batch_fp32_split_error(gpu_lib):
    sets = KB.solver_sets(small_ensemble(n=4, seed=11))
    bt = KB.Batch(sets, "fp32")
    bt.upload_initial()
    dt = bt.timestep()
    bt.step(60)
    outs = bt.download()
    for k, KS in enumerate(sets):
        ref = single(KS, dt[k], 60)
        assert max(rho_u_t_error(outs[k]["prim"], ref["prim"])) < 1e-5


@pytest.mark.parametrize("coll", ["shakhov", "bgk"])
def test_batch_fp32_edge_sizes(gpu_lib, coll):
    """Segment and velocity edge cases of the FP32 segment form: the smallest
    grid (3 cells), a one-segment instance (16 cells), a last segment of one
    cell (17), a last segment of one stepped cell (33), and velocity counts
    that are odd, not a multiple of 4, just above and at the 128 / 256
    boundaries of the thread mapping.  Each instance against its own FP64
    single solve, within 1e-5."""
    cfgs = [KB.shock_config(Ma, nx, nu, coll=coll) for Ma, nx, nu in
            [(1.5, 3, 5), (2.0, 16, 31), (3.0, 17, 128), (4.0, 33, 129), (6.0, 40, 256),
             (1.2, 18, 7)]]
    sets = KB.solver_sets(cfgs)
    bt = KB.Batch(sets, "fp32")
    bt.upload_initial()
    dt = bt.timestep()
    bt.step(40)
    outs = bt.download()
    for k, KS in enumerate(sets):
        ref = single(KS, dt[k], 40)
        assert max(rho_u_t_error(outs[k]["prim"], ref["prim"])) < 1e-5, k


def test_instance_independent_of_batch(gpu_lib):
    cfgs = small_ensemble(n=5, seed=3)
    sets = KB.solver_sets(cfgs)
    full = KB.Batch(sets, "fp64")
    full.upload_initial()
    full.timestep()
    full.step(25)
    alone = KB.Batch([sets[2]], "fp64")
    alone.upload_initial()
    alone.timestep()
    alone.step(25)
    a, b = full.download()[2], alone.download()[0]
    assert np.array_equal(a["prim"], b["prim"]) and np.array_equal(a["h"], b["h"])


def test_converged_instances_stop(gpu_lib):
    sets = KB.solver_sets(small_ensemble(n=3, seed=5))
    bt = KB.Batch(sets, "fp32")
    bt.upload_initial()
    bt.timestep()
    left = bt.run_to_steady(tol=2e-3, max_steps=4000, chunk=100)
    assert left == 0
    s1 = bt.download()
    bt.step(10, tol=2e-3)
    s2 = bt.download()
    for a, b in zip(s1, s2):
        assert np.array_equal(a["h"], b["h"])


BATCH_SHAPES = [(8, 64), (16, 64), (16, 128), (16, 256), (32, 128), (32, 256)]


@pytest.mark.parametrize("seg,threads", BATCH_SHAPES, ids=["s%d-t%d" % s for s in BATCH_SHAPES])
def test_batch_fp32_shapes(gpu_lib, seg, threads):
    """Every shape the autotuner may pick (cells per segment x threads per
    CTA) stays within 1e-5 of the FP64 single solves, incl. instances shorter
    than a segment and last segments of one cell; the persistent grid
    (CTAs looping over segments) gives bit-identical results to one CTA per
    segment."""
    cfgs = [KB.shock_config(Ma, nx, nu) for Ma, nx, nu in
            [(1.5, 3, 5), (2.0, 16, 31), (3.0, 33, 128), (4.0, 65, 129), (6.0, 40, 256),
             (1.2, 9, 7), (2.5, 57, 64)]]
    sets = KB.solver_sets(cfgs)
    outs = {}
    for per in (0, 1):
        bt = KB.Batch(sets, "fp32")
        bt.set_tuning(seg=seg, threads=threads, persist=per)
        assert bt.tuning() == dict(seg=seg, threads=threads, persist=per)
        bt.upload_initial()
        dt = bt.timestep()
        bt.step(40)
        outs[per] = bt.download()
        bt.close()
    for k, KS in enumerate(sets):
        for key in ("w", "prim", "h", "b"):
            assert np.array_equal(outs[0][k][key], outs[1][k][key]), (k, key)
        ref = single(KS, dt[k], 40)
        assert max(rho_u_t_error(outs[0][k]["prim"], ref["prim"])) < 1e-5, k


def test_batch_autotune_picks_a_shape(gpu_lib):
    from kitgpu import tune
    sets = KB.solver_sets(small_ensemble(n=8, seed=3))
    bt = KB.Batch(sets, "fp32")
    bt.upload_initial()
    bt.timestep()
    best, timings = tune.autotune_batch(bt, steps=20, use_cache=False)
    assert (best["seg"], best["threads"]) in BATCH_SHAPES and best["persist"] in (0, 1)
    assert len(timings) == 2 * len(BATCH_SHAPES)
    assert bt.tuning() == best


@pytest.mark.parametrize("coll", ["bgk", "shakhov"])
def test_batch_fp32_high_mach_accuracy(gpu_lib, coll):
    """Mach 6-8 shocks in the FP32 split form, started from the device-built
    equilibrium (kb_batch_init_equilibrium), against the FP64 batch after the
    same 400 steps: rho, U and T within 1e-5.  In the supersonic upstream
    flow the energy is ~35x the thermal energy, so any FP32 rounding that
    reaches w shows up amplified in T = 1 / (2 lambda); the face moments are
    therefore summed from exact product pairs with error-free additions (FP32
    rounding of the moment terms had left T 1e-5 to 5e-5 off after 400
    steps)."""
    cfgs = [KB.shock_config(Ma, nx, nu, coll=coll) for Ma, nx, nu in
            [(8.0, 200, 190), (7.5, 120, 104), (6.2, 300, 96)]]
    sets = KB.solver_sets(cfgs)
    outs = {}
    for prec in ("fp32", "fp64"):
        bt = KB.Batch(sets, prec)
        bt.init_initial()
        bt.timestep()
        bt.step(400)
        outs[prec] = bt.download()
        bt.close()
    for k in range(len(sets)):
        e_rho, e_u, e_t = rho_u_t_error(outs["fp32"][k]["prim"], outs["fp64"][k]["prim"])
        assert e_rho < 1e-5 and e_u < 1e-5 and e_t < 1e-5, (k, e_rho, e_u, e_t)
