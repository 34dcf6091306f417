"""Groups of 2D solves advanced by shared launches (kb_group_*): one launch
of each step kernel per step for all members.  A member's result is
bit-identical to the same solve in a group of its own (the same kernels),
through odd chunk lengths, members joining and leaving between chunks, and
members of different sizes, velocity grids and Knudsen numbers; against the
same solve stepped by its own handle (kb_step, separately compiled kernels
of the same arithmetic, whose FMA contraction the compiler may choose
differently) it agrees to FP32 rounding: 1e-7 in rho, U, T."""
import numpy as np
import pytest

import kitgpu
from kitgpu import _native as N
from kitgpu.group import GROUP_SHAPE, Group, groupable
from kitgpu.serve import cavity_request
from kitgpu.setup import solver_set
from kitgpu.solver import Handle, initial_cells, kb_config, wall_states
from cases import cavity, oracle_for, rho_u_t_error

pytestmark = pytest.mark.gpu

KEYS = ("w", "prim", "h", "b")


def _handle(cfg, precision="fp32"):
    KS = solver_set(cfg)
    vs = KS.vs
    h = Handle(kb_config(KS, precision), vs.flat(vs.u), vs.flat(vs.v), vs.flat(vs.weights))
    w, p = initial_cells(KS)
    h.init_equilibrium(w, p)
    for side, prim in enumerate(wall_states(KS)):
        if KS.set.boundary[side] == "maxwell":
            h.set_wall(side, prim)
    h.set_tuning(**GROUP_SHAPE)
    dt = h.timestep(KS.set.cfl, 0.0, KS.set.maxTime)
    return KS, h, dt


CFGS = [cavity_request(13, 14, 0.075), cavity_request(24, 20, 3e-3), cavity_request(17, 12, 0.5),
        cavity_request(40, 16, 1e-4)]


def _alone(cfg, nsteps):
    """The solve in a group of its own, in the same chunks."""
    KS, h, dt = _handle(cfg)
    g = Group(1)
    g.add(h, dt)
    left, res = nsteps, None
    for n in (5, 7) if nsteps == 12 else (nsteps,):
        g.step_async(n)
        res, _ = g.wait()
        left -= n
    assert left == 0
    g.remove(h)
    g.close()
    out = h.download()
    h.close()
    return out, res[0]


def _own_handle(cfg, nsteps):
    """The solve stepped by its own handle (kb_step)."""
    KS, h, dt = _handle(cfg)
    h.step(dt, nsteps)
    out = h.download()
    h.close()
    return out


@pytest.mark.parametrize("coll", ["shakhov", "bgk"])
def test_group_members_equal_alone(gpu_lib, coll):
    cfgs = [dict(c, collision=coll) for c in CFGS]
    g = Group(8)
    hs = []
    for c in cfgs:
        KS, h, dt = _handle(c)
        assert groupable(h)
        g.add(h, dt)
        hs.append(h)
    for n in (5, 7):  # odd chunks: the members' buffer index alternates
        g.step_async(n)
        res, st = g.wait()
        assert np.all(st == N.KB_OK)
    assert g.launches() > 0
    for k, c in enumerate(cfgs):
        ref, rres = _alone(c, 12)
        got = hs[k].download()
        for key in KEYS:
            assert np.array_equal(got[key], ref[key]), (k, key)
        assert np.array_equal(res[k], rres), k
        own = _own_handle(c, 12)
        assert max(rho_u_t_error(got["prim"], own["prim"])) < 1e-7, k
    g.close()


def test_group_join_and_leave(gpu_lib):
    """A joins; after 6 steps B joins; after 6 more A leaves; B takes 4 more
    (10 in all): A equals 12 steps alone, B 10 steps alone, bit for bit; A
    can be stepped on its own after leaving."""
    g = Group(4)
    KA, A, dtA = _handle(CFGS[0])
    KB_, B, dtB = _handle(CFGS[1])
    g.add(A, dtA)
    g.step_async(6)
    g.wait()
    g.add(B, dtB)
    g.step_async(6)
    g.wait()
    g.remove(A)
    g.step_async(4)
    g.wait()
    refA, _ = _alone(CFGS[0], 12)  # chunking does not change the steps
    refB, _ = _alone(CFGS[1], 10)
    gotA, gotB = A.download(), B.download()
    for key in KEYS:
        assert np.array_equal(gotA[key], refA[key]), key
        assert np.array_equal(gotB[key], refB[key]), key
    A.step(dtA, 3)  # on its own again
    refA3 = _own_handle(CFGS[0], 15)
    assert max(rho_u_t_error(A.download()["prim"], refA3["prim"])) < 1e-7
    g.close()


def test_group_member_against_oracle(gpu_lib):
    """A member stepped 30 steps in a group stays within 1e-5 of the FP64
    oracle in rho, U, T (the FP32 split form's bound)."""
    cfg = cavity(nx=13, ny=11, nu=14, nv=16)
    KS = solver_set(cfg)
    _, h, dt = _handle(cfg)
    g = Group(2)
    g.add(h, dt)
    orc = oracle_for(KS)
    g.step_async(30)
    g.wait()
    orc.step(dt, 30)
    e = rho_u_t_error(h.download()["prim"], orc.get_state()[1])
    assert max(e) < 1e-5, e
    g.close()


def test_group_refuses_uncovered_solves(gpu_lib):
    g = Group(2)
    _, h64, dt = _handle(CFGS[0], precision="fp64")
    assert not groupable(h64)
    with pytest.raises(kitgpu.KitGPUError):
        g.add(h64, dt)
    _, hk, dt = _handle(dict(CFGS[0], flux="kfvs"))
    with pytest.raises(kitgpu.KitGPUError):
        g.add(hk, dt)
    _, hs, dt = _handle(CFGS[0])
    g.add(hs, dt)
    _, hb, dt2 = _handle(dict(CFGS[1], collision="bgk"))
    with pytest.raises(kitgpu.KitGPUError):  # one collision model per group
        g.add(hb, dt2)
    with pytest.raises(kitgpu.KitGPUError):
        g.add(hs, dt)  # already a member
    g.step_async(2)
    with pytest.raises(kitgpu.KitGPUError):  # membership changes wait for the chunk
        g.remove(hs)
    g.wait()
    g.remove(hs)
    g.close()
