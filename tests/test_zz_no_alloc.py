"""kb_timestep_noalloc: the CFL rate computed from the caller's own device
memory without any allocation, for hosts that cannot call cudaMalloc (their
device memory belongs to their own pool or is fully accounted).  Its result
must equal kb_timestep's on the same state, on two calls in a row: the second
call reuses the same fixed scratch with fewer blocks than the first, so
leftovers from the first call would show up as a wrong answer.

This file is collected last on purpose: a run that stops at the first
failure has executed every other test before reaching it.
"""
import ctypes

import numpy as np
import pytest

import kitgpu
from kitgpu import _native as N
from cases import quadrant, sod

pytestmark = pytest.mark.gpu


def noalloc_tmax(handle, prim):
    import torch
    d_prim = torch.tensor(np.ascontiguousarray(prim), dtype=torch.float64, device="cuda")
    d_out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = N.load().kb_timestep_noalloc(ctypes.byref(handle.cfg), d_prim.data_ptr(),
                                      d_out.data_ptr(), stream)
    assert rc == 0, N.load().kb_last_error()
    torch.cuda.synchronize()
    return float(d_out.item())


def test_noalloc_timestep_matches_kb_timestep_twice(gpu_lib):
    # call 1: a 2D state large enough for many scratch blocks and fast flow
    KS1, ctr1, a1, b1, t1 = kitgpu.initialize(quadrant(nx=300, ny=260, nu=8, nv=8))
    h1 = ctr1.handle
    cfl = KS1.set.cfl
    dt_ref = h1.timestep(cfl, 0.0, 1e9)
    tmax = noalloc_tmax(h1, h1.download(("prim",))["prim"])
    assert cfl / tmax == pytest.approx(dt_ref, rel=1e-14)
    # call 2: a smaller 1D state (one block) with a smaller rate; stale
    # partial maxima of call 1 would make this answer too large
    KS2, ctr2, f2, t2 = kitgpu.initialize(sod(nx=200, nu=33))
    h2 = ctr2.handle
    dt_ref2 = h2.timestep(KS2.set.cfl, 0.0, 1e9)
    tmax2 = noalloc_tmax(h2, h2.download(("prim",))["prim"])
    assert KS2.set.cfl / tmax2 == pytest.approx(dt_ref2, rel=1e-14)
    assert tmax2 < tmax
    # and once more on the first state after a few steps (state changed)
    h1.step(dt_ref, 3)
    dt3 = h1.timestep(cfl, 0.0, 1e9)
    tmax3 = noalloc_tmax(h1, h1.download(("prim",))["prim"])
    assert cfl / tmax3 == pytest.approx(dt3, rel=1e-14)


def test_noalloc_allocates_no_device_memory(gpu_lib):
    """After the first call (which loads the module and looks up the scratch
    address), further calls on grids of any allowed size leave the device's
    free memory unchanged."""
    import torch
    KS, ctr, a, b, t = kitgpu.initialize(quadrant(nx=40, ny=30, nu=4, nv=4))
    hd = ctr.handle
    prim = hd.download(("prim",))["prim"]
    d_prim = torch.tensor(prim, dtype=torch.float64, device="cuda")
    d_out = torch.zeros(1, dtype=torch.float64, device="cuda")
    big = torch.ones((1448 * 1448, 4), dtype=torch.float64, device="cuda")  # ~2.1M cells
    lib = N.load()
    stream = torch.cuda.current_stream().cuda_stream
    cfg_big = N.KbConfig()
    ctypes.memmove(ctypes.byref(cfg_big), ctypes.byref(hd.cfg), ctypes.sizeof(cfg_big))
    cfg_big.nx, cfg_big.ny, cfg_big.ngx, cfg_big.ngy = 1448, 1448, 0, 0
    assert lib.kb_timestep_noalloc(ctypes.byref(hd.cfg), d_prim.data_ptr(), d_out.data_ptr(),
                                   stream) == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert lib.kb_timestep_noalloc(ctypes.byref(cfg_big), big.data_ptr(), d_out.data_ptr(),
                                       stream) == 0
        assert lib.kb_timestep_noalloc(ctypes.byref(hd.cfg), d_prim.data_ptr(), d_out.data_ptr(),
                                       stream) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert KS.set.cfl / float(d_out.item()) == pytest.approx(
        hd.timestep(KS.set.cfl, 0.0, 1e9), rel=1e-14)


def test_noalloc_rejects_oversized_grid(gpu_lib):
    KS, ctr, a, b, t = kitgpu.initialize(quadrant(nx=8, ny=8, nu=4, nv=4))
    cfg = N.KbConfig()
    ctypes.memmove(ctypes.byref(cfg), ctypes.byref(ctr.handle.cfg), ctypes.sizeof(cfg))
    cfg.nx, cfg.ny = 2048, 2048  # 4.2M cells > KB_NOALLOC_MAX_CELLS
    rc = N.load().kb_timestep_noalloc(ctypes.byref(cfg), ctypes.c_void_p(1), ctypes.c_void_p(1),
                                      None)
    assert rc == -1
    assert "KB_NOALLOC_MAX_CELLS" in N.load().kb_last_error().decode()
