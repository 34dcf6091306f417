"""Bounded device waits, on the GPU and without a fault.

Every staging kernel waits on mbarriers for its bulk / TMA copies through one
bounded wait; a wait that runs out sets a status bit, the kernel returns, and
the host reports KB_ERR_TIMEOUT instead of hanging the GPU.  kb_wait_probe
makes that wait run out on purpose (a barrier phase nothing completes) with a
short limit.  The test checks that the call returns KB_ERR_TIMEOUT with the
status bit the staging kernels use, that the wait lasted about its limit, and
that the context is still usable: a solve stepped afterwards still equals the
oracle to 1e-12.
"""
import ctypes

import pytest

import kitgpu
from kitgpu import _native as N
from cases import oracle_for, rho_u_t_error, sod

pytestmark = pytest.mark.gpu

LIMIT_S = 0.05


def _probe(lib, limit):
    st = ctypes.c_int32(-1)
    waited = ctypes.c_double(-1.0)
    rc = lib.kb_wait_probe(limit, ctypes.byref(st), ctypes.byref(waited))
    return rc, st.value, waited.value


def test_wait_gives_up_and_context_survives(gpu_lib):
    lib = gpu_lib
    for _ in range(2):  # twice in a row: nothing is left behind by the first
        rc, st, waited = _probe(lib, LIMIT_S)
        assert rc == N.KB_ERR_TIMEOUT, lib.kb_last_error().decode()
        assert st == 2
        assert LIMIT_S <= waited < LIMIT_S + 0.5
    # the same context still computes: a short Sod solve against the oracle
    KS, ctr, face, t = kitgpu.initialize(sod(nx=24, nu=17))
    orc = oracle_for(KS)
    dt = kitgpu.timestep(KS, ctr, 0.0)
    kitgpu.step(KS, ctr, dt, 5)
    orc.step(dt, 5)
    got = ctr.handle.download(("prim",))["prim"]
    assert max(rho_u_t_error(got, orc.get_state()[1])) < 1e-12
    assert ctr.handle.status() == N.KB_OK


def test_probe_rejects_bad_limits(gpu_lib):
    for bad in (0.0, -1.0, 3.0):
        rc, _, _ = _probe(gpu_lib, bad)
        assert rc == N.KB_ERR_ARG
