"""Shared problem builders for the parity tests: one config dict, from which
libkitgpu (through the product's set-up) and the oracle (through its own
restated set-up, oracle/oracle_setup.py) each build their initial state,
walls and velocity tables."""
import numpy as np

import kitgpu
import oracle as O
import oracle_setup as OP


def sod(nx=40, nu=33, flux="kfvs", coll="shakhov", bc="fix", ng=0, Kn=1e-4, maxTime=0.2,
        interp=2, vmesh="newton", omega=0.81):
    return dict(matter="gas", case="sod", space="1d2f1v", flux=flux, collision=coll,
                nSpecies=1, interpOrder=interp, limiter="vanleer", boundary=bc, cfl=0.5,
                maxTime=maxTime, x0=0.0, x1=1.0, nx=nx, nxg=ng, umin=-5.0, umax=5.0, nu=nu,
                vMeshType=vmesh, knudsen=Kn, mach=0.0, prandtl=2 / 3, inK=2.0, omega=omega,
                alphaRef=1.0, omegaRef=0.5)


def shock(nx=40, nu=32, Ma=2.0, flux="kfvs", coll="shakhov", bc="fix", ng=2, Kn=1.0):
    return dict(matter="gas", case="shock", space="1d2f1v", flux=flux, collision=coll,
                nSpecies=1, interpOrder=2, limiter="vanleer", boundary=bc, cfl=0.5,
                maxTime=1.0, x0=-35.0, x1=35.0, nx=nx, nxg=ng, umin=-(5 + 2 * Ma),
                umax=5 + 2 * Ma, nu=nu, vMeshType="rectangle", knudsen=Kn, mach=Ma,
                prandtl=2 / 3, inK=2.0, omega=0.72, alphaRef=1.0, omegaRef=0.5)


def cavity(nx=8, ny=8, nu=12, nv=12, flux="kcu", coll="shakhov", bc="maxwell", ng=0, Kn=0.075,
           vmesh="newton", lid=0.15):
    return dict(matter="gas", case="cavity", space="2d2f2v", flux=flux, collision=coll,
                nSpecies=1, interpOrder=2, limiter="vanleer", boundary=bc, cfl=0.8,
                maxTime=1.0, x0=0.0, x1=1.0, nx=nx, nxg=ng, y0=0.0, y1=1.0, ny=ny, nyg=ng,
                umin=-5.0, umax=5.0, nu=nu, vmin=-5.0, vmax=5.0, nv=nv, vMeshType=vmesh,
                knudsen=Kn, mach=0.0, prandtl=2 / 3, inK=1.0, omega=0.72, alphaRef=1.0,
                omegaRef=0.5, uLid=lid, vLid=0.0, tLid=1.0)


def quadrant(nx=8, ny=8, nu=12, nv=12, flux="ugks", coll="bgk", bc="extra", ng=1, Kn=1e-3,
             seed=20261203):
    return dict(matter="gas", case="quadrant", space="2d2f2v", flux=flux, collision=coll,
                nSpecies=1, interpOrder=2, limiter="vanleer", boundary=bc, cfl=0.5,
                maxTime=1.0, x0=0.0, x1=1.0, nx=nx, nxg=ng, y0=0.0, y1=1.0, ny=ny, nyg=ng,
                umin=-6.0, umax=6.0, nu=nu, vmin=-6.0, vmax=6.0, nv=nv, vMeshType="newton",
                knudsen=Kn, mach=0.0, prandtl=2 / 3, inK=1.0, omega=0.72, alphaRef=1.0,
                omegaRef=0.5)


def oracle_for(KS, threads=None):
    """An oracle solver started from the configuration KS was built from, with
    its own set-up (oracle/oracle_setup.py: velocity grid, gas constants, initial
    cells and walls restated from the reference), not the product's: the GPU
    starts from kitgpu's set-up, so a set-up error on either side shows up as
    a parity failure."""
    P = OP.problem(KS.config, KS.ib_kw)
    orc = O.Oracle(P["cfg"], P["u"], P["v"], P["weights"], threads=threads)
    orc.set_state(P["w"], P["prim"], P["h"], P["b"])
    for side, prim in enumerate(P["walls"]):
        if prim is not None and P["boundary"][side] == "maxwell":
            orc.set_wall(side, prim)
    return orc


def rel(a, b, floor=1e-300):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))) if a.size else 0.0


def rho_u_t_error(pa, pb):
    """Max relative error in rho, U (relative to the local sound speed scale)
    and T = 1 / (2 lambda)."""
    pa, pb = np.asarray(pa), np.asarray(pb)
    nw = pa.shape[-1]
    e_rho = rel(pa[..., 0], pb[..., 0])
    scale = np.sqrt(1.0 / pb[..., -1])
    e_u = float(np.max(np.abs(pa[..., 1:nw - 1] - pb[..., 1:nw - 1]) / scale[..., None]))
    e_t = rel(1.0 / pa[..., -1], 1.0 / pb[..., -1])
    return e_rho, e_u, e_t
