"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py from
the oracle): the oracle reproduces them on this machine (CPU), and the FP64
GPU path matches them within 1e-12 (GPU)."""
import os

import numpy as np
import pytest

import kitgpu
from cases import oracle_for, rho_u_t_error
from golden.make_golden import FIXTURES, run

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(HERE, name + ".npz")))


@pytest.mark.parametrize("name", sorted(FIXTURES))
def test_oracle_reproduces_golden(name):
    g = load(name)
    out = run(name)
    assert out["dt"] == pytest.approx(float(g["dt"]), rel=1e-15)
    e = rho_u_t_error(out["prim"], g["prim"])
    assert max(e) < 1e-13, e
    assert np.max(np.abs(out["h"] - g["h"])) < 1e-13 * np.max(np.abs(g["h"]))


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(FIXTURES))
def test_gpu_fp64_matches_golden(gpu_lib, name):
    cfg, n = FIXTURES[name]
    g = load(name)
    KS, ctr, *faces, t = kitgpu.initialize(cfg)
    dt = kitgpu.timestep(KS, ctr, 0.0)
    assert dt == pytest.approx(float(g["dt"]), rel=1e-14)
    res = kitgpu.step(KS, ctr, dt, n)
    s = ctr.handle.download()
    e = rho_u_t_error(s["prim"], g["prim"])
    assert max(e) < 1e-12, e
    assert np.max(np.abs(s["h"] - g["h"])) < 1e-12 * np.max(np.abs(g["h"]))
    assert np.allclose(res, g["residual"], rtol=1e-9)
