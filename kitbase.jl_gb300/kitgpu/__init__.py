"""kitgpu: GB300-native (sm_103a) discrete-velocity-method time step for
KitBase.jl's 1D2F1V and 2D2F2V solvers.

The compute path is libkitgpu.so (C ABI, include/kitgpu.h); this package is the
host-side mirror of the reference's SolverSet / init_fvm / reconstruct! /
evolve! / update! / solve! API over that ABI.
"""
from ._native import KitGPUError, load  # noqa: F401
from .setup import (IB, Gas, PSpace1D, PSpace2D, Setup, SolverSet, VSpace1D,  # noqa: F401
                    VSpace2D, conserve_prim, gas_property, heat_capacity_ratio, ib_cavity,
                    ib_quadrant, ib_rh, ib_sod, maxwellian, newton_cotes, prim_conserve,
                    read_cfg, read_dict, ref_vhs_vis, rh_states, solver_set)
from .solver import (Cells, Faces, Handle, evolve, extract_sol, init_fvm,  # noqa: F401
                     initial_state, initialize, kb_config, read_checkpoint, reconstruct,
                     solve, step, timestep, update, wall_states, write_checkpoint)

__version__ = "0.1.0"
