"""Generate the golden fixtures in this folder from the FP64 C oracle.

KitBase.jl (Julia) cannot run on the machines this project builds on and its
test suite holds no golden vectors for the DVM step, so these fixtures pin the
oracle's own results (regression across x86_64 / aarch64 builds and over time)
and give the GPU tests a stored answer.  They do not pin the oracle to the
reference; see tests/test_oracle.py for the invariants and known answers that do.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "kitbase.jl_gb300"), os.path.join(ROOT, "oracle"),
          os.path.join(ROOT, "tests")):
    sys.path.insert(0, p)

import kitgpu  # noqa: E402
from cases import cavity, oracle_for, quadrant, sod  # noqa: E402

FIXTURES = {
    "sod_kfvs_shakhov_40x33": (sod(nx=40, nu=33, flux="kfvs", coll="shakhov"), 30),
    "sod_kcu_maxwell_40x33": (sod(nx=40, nu=33, flux="kcu", coll="bgk", bc="maxwell"), 30),
    "sod_ugks_extra_40x33": (sod(nx=40, nu=33, flux="ugks", coll="shakhov", bc="extra", ng=1,
                                 Kn=1e-2), 30),
    "cavity_kcu_shakhov_8x8x12x12": (cavity(), 6),
    "quadrant_ugks_bgk_8x8x12x12": (quadrant(), 6),
}


def run(name):
    cfg, n = FIXTURES[name]
    KS = kitgpu.solver_set(cfg)
    orc = oracle_for(KS, threads=1)
    dt = orc.timestep(KS.set.cfl, 0.0, KS.set.maxTime)
    res = orc.step(dt, n)
    w, p, h, b = orc.get_state()
    return dict(dt=dt, nsteps=n, residual=res, w=w, prim=p, h=h, b=b)


def main():
    for name in FIXTURES:
        out = run(name)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, out["prim"].shape, "dt=%.6e" % out["dt"])


if __name__ == "__main__":
    main()
