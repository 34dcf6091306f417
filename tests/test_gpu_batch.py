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
