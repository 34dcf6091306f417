"""Checkpoint / restart round trip through the C ABI (the role of write_jld and
initialize("*.jld2"), src/IO/io_write.jl:34-40, src/Solver/solver_init.jl:19-26).

A solve that is checkpointed after K steps, restarted from the file in a new
solver and advanced K more steps must end bit-identical to the same solve
advanced 2K steps without interruption: the checkpoint holds every cell field
the step reads (w, prim, h, b incl. ghosts), and the download / upload
conversions are exact (FP32 values are exact in FP64).
"""
import numpy as np
import pytest

import kitgpu
from cases import cavity, quadrant, sod

pytestmark = pytest.mark.gpu

CASES = [
    ("sod-kfvs-shakhov", sod(), "fp64"),
    ("sod-kcu-maxwell", sod(flux="kcu", bc="maxwell"), "fp32"),
    ("cavity-kcu-shakhov", cavity(nx=12, ny=10, nu=12, nv=14), "fp64"),
    ("cavity-kcu-shakhov-fp32", cavity(nx=12, ny=10, nu=12, nv=14), "fp32"),
    ("quadrant-ugks-bgk-fp32", quadrant(nx=14, ny=13, nu=16, nv=16), "fp32"),
]


@pytest.mark.parametrize("name,cfg,prec", CASES, ids=[c[0] for c in CASES])
def test_restart_is_bit_identical(gpu_lib, tmp_path, name, cfg, prec):
    K = 7
    KS, ctr, *faces, t = kitgpu.initialize(cfg, precision=prec)
    dt = kitgpu.timestep(KS, ctr, 0.0)
    kitgpu.step(KS, ctr, dt, K)
    path = str(tmp_path / "ckpt.npz")
    kitgpu.write_checkpoint(path, KS, ctr, K * dt, slopes=True)
    kitgpu.step(KS, ctr, dt, K)
    ref = ctr.handle.download()

    KS2, ctr2, *faces2, t2 = kitgpu.initialize(path)
    assert t2 == K * dt
    assert ctr2.handle.cfg.precision == ctr.handle.cfg.precision
    kitgpu.step(KS2, ctr2, dt, K)
    got = ctr2.handle.download()
    for k in ("w", "prim", "h", "b"):
        assert np.array_equal(got[k], ref[k]), k


def test_checkpoint_fields(gpu_lib, tmp_path):
    """The file carries the ControlVolume2F fields per cell with the
    reference's shapes: h[u, v] per cell (column-major, so (nv, nu) here),
    slopes with the direction as their own axis."""
    cfg = cavity(nx=6, ny=5, nu=8, nv=10, ng=1)
    KS, ctr, *faces, t = kitgpu.initialize(cfg)
    path = str(tmp_path / "c.npz")
    kitgpu.write_checkpoint(path, KS, ctr, 0.25, slopes=True)
    d = np.load(path)
    ncell = 8 * 7
    assert d["ctr.w"].shape == (ncell, 4) and d["ctr.prim"].shape == (ncell, 4)
    assert d["ctr.h"].shape == (ncell, 10, 8) and d["ctr.b"].shape == (ncell, 10, 8)
    assert d["ctr.sw"].shape == (ncell, 2, 4) and d["ctr.sh"].shape == (ncell, 2, 10, 8)
    assert list(d["cells"]) == [8, 7] and list(d["ghosts"]) == [1, 1]
    c = ctr[3, 2]  # 1-based cell (3, 2) of the OffsetArray
    ci = (2 - 1 + 1) * 8 + (3 - 1 + 1)
    assert np.array_equal(d["ctr.h"][ci].T, c.h)
    assert float(d["t"]) == 0.25


def test_checkpoint_shape_mismatch_raises(gpu_lib, tmp_path):
    KS, ctr, face, t = kitgpu.initialize(sod(nx=20))
    path = str(tmp_path / "s.npz")
    kitgpu.write_checkpoint(path, KS, ctr, 0.0)
    KS2, ctr2, face2, t2 = kitgpu.initialize(sod(nx=21))
    with pytest.raises(ValueError):
        kitgpu.read_checkpoint(path, ctr2)


PIN_CASES = [
    ("sod-rows", sod(), "fp32"),                                   # 101 velocities: padded rows
    ("cavity-dense", cavity(nx=12, ny=10, nu=12, nv=14), "fp32"),  # 168: dense pairs
    ("cavity-dense-fp64", cavity(nx=12, ny=10, nu=12, nv=14), "fp64"),
    ("quadrant-dense", quadrant(nx=14, ny=13, nu=16, nv=16), "fp32"),
]


@pytest.mark.parametrize("name,cfg,prec", PIN_CASES, ids=[c[0] for c in PIN_CASES])
@pytest.mark.parametrize("offset", [0, 1], ids=["aligned", "offset8"])
def test_pinned_transfers_match_pageable(gpu_lib, name, cfg, prec, offset):
    """Page-locked host arrays are converted in place over the host link
    (dense pairs when the rows are unpadded and 16-byte aligned, padded rows
    otherwise); download and upload through them equal the pageable path,
    which goes through the device staging buffer, bit for bit."""
    import torch
    from kitgpu import _native as N
    KS, ctr, *faces, t = kitgpu.initialize(cfg, precision=prec)
    hd = ctr.handle
    dt = kitgpu.timestep(KS, ctr, 0.0)
    kitgpu.step(KS, ctr, dt, 5)
    ref = hd.download()

    def pinned(shape):
        n = int(np.prod(shape))
        buf = torch.zeros(n + offset, dtype=torch.float64, pin_memory=True).numpy()
        return buf[offset:].reshape(shape)

    h, b = pinned(ref["h"].shape), pinned(ref["b"].shape)
    w, p = np.zeros_like(ref["w"]), np.zeros_like(ref["prim"])
    hd.call("kb_download_state", N.ptr(w), N.ptr(p), N.ptr(h), N.ptr(b))
    assert np.array_equal(h, ref["h"]) and np.array_equal(b, ref["b"])

    # upload the pinned copy (perturbed, so the upload is seen) and compare
    # with the same values uploaded from pageable arrays into a second solve
    h *= 1.0 + 1e-3
    KS2, ctr2, *faces2, t2 = kitgpu.initialize(cfg, precision=prec)
    hd.call("kb_upload_state", N.ptr(ref["w"]), N.ptr(ref["prim"]), N.ptr(h), N.ptr(b))
    ctr2.handle.upload(ref["w"], ref["prim"], np.array(h), np.array(b))
    got, want = hd.download(), ctr2.handle.download()
    for k in ("h", "b"):
        assert np.array_equal(got[k], want[k]), k
    kitgpu.step(KS, ctr, dt, 3)
    kitgpu.step(KS2, ctr2, dt, 3)
    got, want = hd.download(), ctr2.handle.download()
    for k in ("w", "prim", "h", "b"):
        assert np.array_equal(got[k], want[k]), k
