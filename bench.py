"""Benchmark of the GB300 DVM time step (driver contract: one JSON line).

Workload: the four-quadrant 2D2F2V solve sized for the HBM roofline -- 512 x 512
cells, 64 x 64 Newton-Cotes velocities on [-6, 6]^2, UGKS flux, BGK relaxation,
Kn = 1e-3, extrapolation boundaries with one ghost layer, seeded quadrant states
(rho ~ U(0.1, 1.5), U, V ~ U(-0.5, 0.5), lambda ~ U(0.4, 1.2)).  One step =
reconstruct! + evolve! + update! over all 1.07e9 cell-velocity points.

  value      cell-velocity updates/s of the FP32-split form (FP32 h / b, FP64
             moments, w, prim), state resident in HBM, CUDA events on the
             library's stream; inputs (17 GB of state) are larger than L2.
  e2e        the same through the C ABI with host buffers: upload of the FP64
             host state from pinned memory, K steps, download of the state.
  roofline   pass B (pointwise update, the dominant kernel): algorithmic bytes
             (read h, b once + write h, b once = 16 B per cell-velocity in FP32)
             / its CUDA-event time, against the measured HBM copy bandwidth.
  fp64_plain the plain FP64 GPU path on the same workload.
  cpu_baseline  the FP64 C oracle (restatement of the Julia reference; Julia
             is not available) on a bounded sample with all host threads.

--impl reference times that CPU restatement alone on the same metric.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "kitbase.jl_gb300"))

WORKLOAD = dict(nx=512, ny=512, nu=64, nv=64, umax=6.0, Kn=1e-3, flux="ugks", coll="bgk",
                bc="extra", ng=1, seed=20261203, cfl=0.5)
METRIC = "DVM cell-velocity updates/s"
UNIT = "cell-velocity updates/s"


def quadrant_cfg(nx, ny, nu, nv, umax, Kn, flux, coll, bc, ng, seed, cfl, **_):
    return dict(matter="gas", case="quadrant", space="2d2f2v", flux=flux, collision=coll,
                nSpecies=1, interpOrder=2, limiter="vanleer", boundary=bc, cfl=cfl, maxTime=1.0,
                x0=0.0, x1=1.0, nx=nx, nxg=ng, y0=0.0, y1=1.0, ny=ny, nyg=ng, umin=-umax,
                umax=umax, nu=nu, vmin=-umax, vmax=umax, nv=nv, vMeshType="newton", knudsen=Kn,
                mach=0.0, prandtl=2.0 / 3.0, inK=1.0, omega=0.81, alphaRef=1.0, omegaRef=0.5)


def quadrant_state(KS, out_h=None, out_b=None):
    """Vectorised init_fvm state of the quadrant preset (all cells incl. ghosts)."""
    import kitgpu
    ps, gas, vs = KS.ps, KS.gas, KS.vs
    xm, ym = (ps.x0 + ps.x1) / 2, (ps.y0 + ps.y1) / 2
    X = ps.x.T.ravel()  # cell order: x fastest
    Y = ps.y.T.ravel()
    q = np.where(X > xm, np.where(Y > ym, 0, 3), np.where(Y > ym, 1, 2))
    quads = KS.ib.p["quads"]
    W4 = np.array([kitgpu.prim_conserve(p, gas.gamma) for p in quads])
    P4 = np.array([kitgpu.conserve_prim(w, gas.gamma) for w in W4])
    u, v = vs.flat(vs.u), vs.flat(vs.v)
    H4 = np.array([kitgpu.maxwellian(u, p, v) for p in P4])
    B4 = H4 * gas.K / 2.0 / P4[:, -1:]
    n = len(q)
    h = out_h if out_h is not None else np.empty((n, len(u)))
    b = out_b if out_b is not None else np.empty((n, len(u)))
    for k in range(4):
        m = q == k
        h[m] = H4[k]
        b[m] = B4[k]
    return W4[q], P4[q], h, b


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=2)

    def summary(self):
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in self.rows:
            if len(r) >= 9:
                for k, nm in enumerate(names):
                    if r[5 + k].lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if args.impl == "ours" and torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        pg = dist
    return ws, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    if pg.get_backend() == "nccl":
        t = t.cuda()
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def cpu_oracle(threads, nx=64):
    """FP64 oracle on an nx x nx-cell sample of the workload (same velocity grid,
    flux, collision and boundaries): (oracle, dt, cell-velocity points)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import kitgpu
    import oracle as O
    wl = dict(WORKLOAD, nx=nx, ny=nx)
    KS = kitgpu.solver_set(quadrant_cfg(**wl))
    cfg = kitgpu.kb_config(KS)
    c = O.make_config(cfg.dim, cfg.nx, cfg.ny, cfg.ngx, cfg.ngy, cfg.nu, cfg.nv, cfg.flux,
                      cfg.collision, [cfg.bc[k] for k in range(4)], cfg.interp_order, cfg.x0,
                      cfg.x1, cfg.y0, cfg.y1, cfg.umax, cfg.vmax, cfg.K, cfg.gamma, cfg.mu_ref,
                      cfg.omega, cfg.Pr)
    vs = KS.vs
    orc = O.Oracle(c, vs.flat(vs.u), vs.flat(vs.v), vs.flat(vs.weights), threads=threads)
    w, p, h, b = quadrant_state(KS)
    orc.set_state(w, p, h, b)
    dt = orc.timestep(KS.set.cfl, 0.0, KS.set.maxTime)
    return orc, dt, nx * nx * vs.nu * vs.nv


def cpu_sample(threads, nsteps=None, nx=64):
    """Oracle throughput on the sample: (updates/s, description, s per step)."""
    orc, dt, cv = cpu_oracle(threads, nx)
    orc.step(dt, 1)  # warm-up (page faults, thread pool)
    if nsteps is None:
        t0 = time.perf_counter()
        orc.step(dt, 1)
        one = time.perf_counter() - t0
        nsteps = max(1, int(15.0 / max(one, 1e-3)))
    t0 = time.perf_counter()
    orc.step(dt, nsteps)
    el = time.perf_counter() - t0
    desc = ("%dx%d-cell sample of the workload (64x64 velocities, UGKS+BGK), %d step(s), "
            "FP64 C oracle with OpenMP" % (nx, nx, nsteps))
    return cv * nsteps / el, desc, el / nsteps


def run_reference(args):
    ws, rank, local, pg = dist_setup(args)
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    import kitgpu  # noqa: F401  (host-side setup only)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    nx = 64
    orc, dt, cv = cpu_oracle(threads, nx)
    for _ in range(args.warmup):
        orc.step(dt, 1)
    t0 = time.perf_counter()
    orc.step(dt, args.steps)
    el = time.perf_counter() - t0
    val = cv * args.steps / el
    desc = ("each step: one DVM step of a %dx%d-cell sample of the workload (64x64 velocities, "
            "UGKS+BGK), FP64 C oracle with OpenMP" % (nx, nx))
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT,
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * el / max(args.steps, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "four-quadrant 2D2F2V 512x512 cells x 64x64 velocities, "
                                   "UGKS + BGK, Kn=1e-3 (each step: a 64x64-cell sample)"},
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": desc + "; Julia KitBase is not installable here, the "
                                              "C restatement of its algorithm stands in"},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


ERROR_CASES = (
    ("sod 1D2F1V 200 cells x 101 velocities, KFVS + Shakhov, Kn=1e-4, to t=0.2",
     dict(matter="gas", case="sod", space="1d2f1v", flux="kfvs", collision="shakhov", nSpecies=1,
          interpOrder=2, limiter="vanleer", boundary="fix", cfl=0.5, maxTime=0.2, x0=0.0,
          x1=1.0, nx=200, nxg=0, umin=-5.0, umax=5.0, nu=101, vMeshType="newton",
          knudsen=1e-4, mach=0.0, prandtl=2.0 / 3.0, inK=2.0, omega=0.81, alphaRef=1.0,
          omegaRef=0.5), None),
    ("cavity 2D2F2V 64^2 cells x 28^2 velocities, KCU + Shakhov, Kn=0.075, Maxwell walls, "
     "lid 0.15, 2000 steps",
     dict(matter="gas", case="cavity", space="2d2f2v", flux="kcu", collision="shakhov",
          nSpecies=1, interpOrder=2, limiter="vanleer", boundary="maxwell", cfl=0.8,
          maxTime=1.0, x0=0.0, x1=1.0, nx=64, nxg=0, y0=0.0, y1=1.0, ny=64, nyg=0, umin=-5.0,
          umax=5.0, nu=28, vmin=-5.0, vmax=5.0, nv=28, vMeshType="newton", knudsen=0.075,
          mach=0.0, prandtl=2.0 / 3.0, inK=1.0, omega=0.72, alphaRef=1.0, omegaRef=0.5,
          uLid=0.15, vLid=0.0, tLid=1.0), 2000),
    ("four-quadrant 2D2F2V 128^2 cells x 64^2 velocities, UGKS + BGK, Kn=1e-3, 40 steps",
     "quadrant128", 40),
)


def error_table(args):
    """L-inf of the FP32-split form against the plain FP64 GPU path after the
    same steps: rho, U, T (prim_errors) and q relative to max |q|; and the
    throughput of both forms on these runs (C1 Sod and C2 cavity in full,
    the C3 physics at 128^2): the steps are timed on the host around the
    synchronous kb_step (eager launches, no graph)."""
    import kitgpu
    rows = []
    for name, cfg, nsteps in ERROR_CASES:
        if cfg == "quadrant128":
            cfg = quadrant_cfg(**dict(WORKLOAD, nx=128, ny=128))
        KS = kitgpu.solver_set(cfg)
        outs, rate, msps = {}, {}, {}
        for prec in ("fp32", "fp64"):
            ctr = kitgpu.init_fvm(KS, prec)[0]
            dt = kitgpu.timestep(KS, ctr, 0.0)
            n = nsteps or int(np.floor(KS.set.maxTime / dt)) + 1
            t0 = time.perf_counter()
            kitgpu.step(KS, ctr, dt, n)
            el = time.perf_counter() - t0
            c = ctr.handle.cfg
            cv = c.nx * (c.ny if KS.dim == 2 else 1) * ctr.handle.nvel
            rate[prec] = cv * n / el
            msps[prec] = 1e3 * el / n
            outs[prec] = ctr.handle.download()
            ctr.handle.close()
        vs = KS.vs
        u, v, wt = ((vs.u, None, vs.weights) if KS.dim == 1
                    else (vs.flat(vs.u), vs.flat(vs.v), vs.flat(vs.weights)))
        e = prim_errors(outs["fp32"]["prim"], outs["fp64"]["prim"])
        qa, qb = heat_flux(outs["fp32"], u, v, wt), heat_flux(outs["fp64"], u, v, wt)
        eq = float(np.max(np.abs(qa - qb)) / max(np.max(np.abs(qb)), 1e-300))
        wa, wb = outs["fp32"]["w"], outs["fp64"]["w"]
        rows.append({"case": name, "steps": n, "rho": e[0], "U": e[1], "T": e[2],
                     "q_rel_to_max": eq,
                     "cv_per_s": rate, "ms_per_step": msps,
                     "speedup_fp32_vs_fp64": rate["fp32"] / rate["fp64"],
                     "mass_fp32_vs_fp64": float(abs(wa[:, 0].sum() - wb[:, 0].sum())
                                                / wb[:, 0].sum())})
    return {"reference": "plain FP64 GPU path (held to the FP64 oracle within 1e-12 by the "
                         "parity tests)", "cases": rows}


def run_ours(args):
    import torch
    ws, rank, local, pg = dist_setup(args)
    torch.cuda.set_device(local)
    import kitgpu
    from kitgpu import _native as N
    kitgpu.load()

    wl = dict(WORKLOAD)
    if args.small:
        wl.update(nx=128, ny=128)
    KS = kitgpu.solver_set(quadrant_cfg(**wl))
    vs = KS.vs
    ncell_phys = wl["nx"] * wl["ny"]
    nvel = vs.nu * vs.nv
    cv = ncell_phys * nvel  # cell-velocity updates per step
    nxt, nyt = wl["nx"] + 2 * wl["ng"], wl["ny"] + 2 * wl["ng"]
    ncell = nxt * nyt

    # pinned host state (FP64, the reference's storage type)
    pin = lambda shape: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    h_host, b_host = pin((ncell, nvel)), pin((ncell, nvel))
    w_host, p_host, _, _ = quadrant_state(KS, h_host, b_host)
    w_host = np.ascontiguousarray(w_host)
    p_host = np.ascontiguousarray(p_host)
    h_out, b_out = pin((ncell, nvel)), pin((ncell, nvel))
    w_out, p_out = np.zeros_like(w_host), np.zeros_like(p_host)

    def make(prec, tuning=None):
        hd = kitgpu.Handle(kitgpu.kb_config(KS, prec), vs.flat(vs.u), vs.flat(vs.v),
                           vs.flat(vs.weights))
        hd.upload(w_host, p_host, h_host, b_host)
        if tuning:
            hd.set_tuning(**tuning)
        return hd

    hd = make("fp32")
    dt = hd.timestep(KS.set.cfl, 0.0, KS.set.maxTime)
    # launch shapes from the project autotuner (advances the state a few steps;
    # the state is re-uploaded before timing)
    from kitgpu import tune
    best, _ = tune.autotune(hd, dt, steps=1, use_cache=not args.retune)
    hd.upload(w_host, p_host, h_host, b_host)
    stream = torch.cuda.ExternalStream(hd.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    hd.step(dt, args.warmup)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    n0 = hd.launches()
    barrier(pg)
    torch.cuda.synchronize()
    ev0.record(stream)
    hd.step(dt, args.steps)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(pg)
    ms = ev0.elapsed_time(ev1)
    launches = hd.launches() - n0
    clocks.stop()
    ms = max_over_ranks(pg, ms)
    value = cv * args.steps * ws / (ms / 1e3)

    # per-stage kernel times (events around each kernel group) for the roofline
    hd.set_timing(True)
    nprof = max(2, min(args.steps, 5))
    hd.step(dt, nprof)
    st = hd.timing()
    hd.set_timing(False)
    upd_ms = st["update"][0] / st["update"][1]
    mom_ms = st["moments"][0] / st["moments"][1]
    step_ms = sum(v[0] for v in st.values()) / nprof
    peak, peak_kind = measured_peaks()
    alg_b = 16.0 * cv  # read h, b once + write h, b once, FP32
    achieved = alg_b / (upd_ms / 1e3) / 1e9
    # pass-B kernel of the tuned shape; DRAM traffic per launch from the
    # committed ncu capture of that kernel, scaled by the cv of a launch
    pair = best.get("march_bs") == 64
    kname = ("k_march4 (pass B, two velocities per thread, TMA row ring)" if pair
             else "k_march3 (pass B, one velocity per thread, TMA row ring)")
    traffic = None
    tp = os.path.join(ROOT, "profiles", "k_march4_traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            tt = json.load(f)
        if all(best.get(k) == v for k, v in tt.get("tuning", {}).items()):
            traffic = tt.get("bytes_per_cv", 0) * cv or None

    # end to end through the C ABI: pinned host state in, K steps, state out
    barrier(pg)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hd.upload(w_host, p_host, h_host, b_host)
    hd.step(dt, args.steps)
    hd.call("kb_download_state", N.ptr(w_out), N.ptr(p_out), N.ptr(h_out), N.ptr(b_out))
    e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(pg, e2e_s)
    h2d = (w_host.nbytes + p_host.nbytes + h_host.nbytes + b_host.nbytes) / args.steps
    d2h = (w_out.nbytes + p_out.nbytes + h_out.nbytes + b_out.nbytes) / args.steps
    e2e_val = cv * args.steps * ws / e2e_s
    hd.close()

    # plain FP64 GPU path on the same workload
    fp64 = None
    if not args.no_fp64:
        h64 = make("fp64")
        h64.step(dt, 1)
        k64 = max(1, min(args.steps, 3))
        torch.cuda.synchronize()
        s64 = torch.cuda.ExternalStream(h64.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s64)
        h64.step(dt, k64)
        e1.record(s64)
        torch.cuda.synchronize()
        ms64 = max_over_ranks(pg, e0.elapsed_time(e1))
        v64 = cv * k64 * ws / (ms64 / 1e3)
        h64.set_timing(True)
        h64.step(dt, 1)
        t64 = h64.timing()
        h64.close()
        u64 = t64["update"][0] / t64["update"][1]
        fp64 = {"value": v64, "unit": UNIT, "steps": k64, "ms_per_step": ms64 / k64,
                "speedup_fp32_split": value / v64,
                "roofline": {"bound": "hbm", "achieved": 32.0 * cv / (u64 / 1e3) / 1e9,
                             "peak": peak, "unit": "GB/s",
                             "frac": 32.0 * cv / (u64 / 1e3) / 1e9 / peak},
                "stage_ms": {k: v[0] / max(v[1], 1) for k, v in t64.items()}}

    # L-inf error of the FP32-split form against the plain FP64 GPU path (which
    # the parity tests hold to the FP64 oracle within 1e-12) on the small
    # configurations at full size and on the headline physics at 128^2 cells
    err = None
    if not args.no_error and rank == 0:
        err = error_table(args)

    cpu = None
    if rank == 0 and not args.no_cpu:
        thr = os.cpu_count() or 1
        v, desc, per = cpu_sample(thr)
        cpu = {"value": v, "unit": UNIT, "cores": thr, "kind": "port", "sample": desc}

    if rank != 0:
        return 0
    blocks = {}
    if not args.no_batch:
        blocks["batch"] = batch_block(args, peak)
    if not args.no_serve:
        blocks["serve"] = serve_block(args)
    if not args.no_unstruct:
        blocks["unstructured"] = unstruct_block(args, peak)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "precision": "FP32 h, b and pointwise fluxes; FP64 moments (compensated), w, prim, q",
        "data": "synthetic",
        "config": {"workload": "four-quadrant 2D2F2V %dx%d cells x %dx%d velocities on [-6,6]^2, "
                               "UGKS + BGK, Kn=1e-3, extrapolation boundaries"
                               % (wl["nx"], wl["ny"], vs.nu, vs.nv),
                   "cells": ncell_phys, "velocities": nvel, "cell_velocity_per_step": cv,
                   "state_bytes_fp32": 4 * 4 * ncell * nvel,
                   "l2": "inputs larger than L2 (state far above 129 MB), no flush",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "kernel": kname,
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": traffic,
                     "algorithmic_bytes_per_launch": alg_b, "launch_ms": upd_ms},
        "step_roofline": {"achieved": alg_b / (ms / args.steps / 1e3) / 1e9, "unit": "GB/s",
                          "frac": alg_b / (ms / args.steps / 1e3) / 1e9 / peak,
                          "note": "whole step (pass A + pass B + small kernels), 16 B per cv"},
        "stage_ms": {k: v[0] / max(v[1], 1) for k, v in st.items()},
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "note": "kb_upload_state (FP64 pinned host) + K kb_step + kb_download_state"},
        "gpu_launches": launches,
        "tuning": best,
        "clocks": clocks.summary(),
        "fp64_plain": fp64,
        "linf_error_vs_fp64": err,
        "cpu_baseline": cpu,
    }
    line.update(blocks)
    print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()
    return 0


def prim_errors(pa, pb):
    """L-inf of rho (relative), U (against the thermal speed sqrt(1/lambda)) and
    T = 1/(2 lambda) (relative) of prim pa against pb ([..., dim+2])."""
    pa, pb = np.asarray(pa), np.asarray(pb)
    nw = pa.shape[-1]
    e_rho = float(np.max(np.abs(pa[..., 0] - pb[..., 0]) / pb[..., 0]))
    e_u = float(np.max(np.abs(pa[..., 1:nw - 1] - pb[..., 1:nw - 1]) * np.sqrt(pb[..., -1:])))
    e_t = float(np.max(np.abs(1 / pa[..., -1] - 1 / pb[..., -1]) * pb[..., -1]))
    return e_rho, e_u, e_t


def heat_flux(st, u, v, wt):
    """q per cell from h, b (heat_flux 2F1V / 2F2V, src/Theory/theory_moments.jl:530-531,
    :567-578); st holds prim [ncell, nw], h, b [ncell, nvel]."""
    P = st["prim"]
    cu = u[None, :] - P[:, 1:2]
    if v is None:
        return (0.5 * ((wt * cu ** 3 * st["h"]).sum(1) + (wt * cu * st["b"]).sum(1)))[:, None]
    cvv = v[None, :] - P[:, 2:3]
    c2 = cu * cu + cvv * cvv
    q1 = 0.5 * ((wt * cu * c2 * st["h"]).sum(1) + (wt * cu * st["b"]).sum(1))
    q2 = 0.5 * ((wt * cvv * c2 * st["h"]).sum(1) + (wt * cvv * st["b"]).sum(1))
    return np.stack([q1, q2], 1)


def batch_block(args, peak):
    """Batched shock-structure ensemble (512 instances): FP32-split batch step
    (fused launch per step, CUDA graph), its roofline fraction, the run to the
    1e-8 steady residual, L-inf against the FP64 batch after the same steps,
    and the plain FP64 GPU path looped per instance."""
    import torch
    import kitgpu
    from kitgpu import batch as KB
    sets = KB.solver_sets(KB.shock_ensemble(args.instances))
    out = {"workload": "batched ensemble of %d 1D shock-structure solves (Mach U(1.2,8), cells "
                       "U{50..400}, velocities U{48..200} on +-(5+2Ma)), KFVS + Shakhov, Kn=1, "
                       "upstream rho=1, lambda=0.5" % len(sets)}
    states = {}
    from kitgpu import tune
    for prec in ("fp32", "fp64"):
        bt = KB.Batch(sets, prec)
        bt.init_initial()
        bt.timestep()
        tuned, timings = None, None
        if prec == "fp32":
            # kernel shape from the project autotuner (the search advances
            # the state, so the batch restarts from its initial state)
            tuned, timings = tune.autotune_batch(bt, steps=200, use_cache=not args.retune)
            bt.init_initial()
            bt.timestep()
        bt.step(args.warmup)
        cv = bt.cell_velocity_points()
        # an FP32 batch step is ~0.2 ms: time at least 500 of them so the
        # host's launch and synchronisation cost is amortised
        nst = max(args.steps, 500) if prec == "fp32" else max(args.steps, 50)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        bt.step(nst)
        el = time.perf_counter() - t0
        val = cv * nst / el
        esz = 16.0 if prec == "fp32" else 32.0
        out[prec] = {"value": val, "unit": UNIT, "ms_per_step": 1e3 * el / nst, "steps": nst,
                     "cell_velocity_per_step": cv,
                     "roofline": {"bound": "hbm", "achieved": val * esz / 1e9, "peak": peak,
                                  "unit": "GB/s", "frac": val * esz / 1e9 / peak,
                                  "bytes_per_cv": esz}}
        # same number of steps from the initial state in both forms
        bt.init_initial()
        bt.timestep()
        bt.step(args.batch_err_steps)
        states[prec] = bt.download()
        if prec == "fp32":
            bt.init_initial()
            bt.timestep()
            t0 = time.perf_counter()
            left = bt.run_to_steady(tol=1e-8, max_steps=args.max_steady, chunk=500)
            r = bt.residual[:, :3].max(axis=1)
            out["fp32"]["steady"] = {"tol": 1e-8, "steps": bt.steps,
                                     "seconds": time.perf_counter() - t0,
                                     "unconverged": left, "instances": bt.n,
                                     "below_1e-6": int(np.sum(r < 1e-6))}
            out["fp32"]["tuning"] = bt.tuning()
            if timings:
                out["fp32"]["tuning_ms_per_step"] = timings
        bt.close()
    # steady convergence of both forms on the same sample of instances and
    # step cap: the rate of approach to the steady shock, not the storage
    # precision, is what limits it
    sample = sets[:: max(1, len(sets) // args.steady_sample)][: args.steady_sample]
    conv = {}
    for prec in ("fp32", "fp64"):
        bt = KB.Batch(sample, prec)
        bt.init_initial()
        bt.timestep()
        left = bt.run_to_steady(tol=1e-8, max_steps=args.steady_cap, chunk=500)
        r = bt.residual[:, :3].max(axis=1)
        conv[prec] = {"below_1e-8": int(np.sum(r < 1e-8)), "below_1e-6": int(np.sum(r < 1e-6)),
                      "median_residual": float(np.median(r))}
        bt.close()
    out["steady_sample"] = {"instances": len(sample), "steps": args.steady_cap, **conv}
    er = np.zeros(4)
    for K, a, b in zip(sets, states["fp32"], states["fp64"]):
        e = prim_errors(a["prim"], b["prim"])
        qa = heat_flux(a, K.vs.u, None, K.vs.weights)
        qb = heat_flux(b, K.vs.u, None, K.vs.weights)
        eq = float(np.max(np.abs(qa - qb)) / max(np.max(np.abs(qb)), 1e-300))
        er = np.maximum(er, list(e) + [eq])
    out["linf_fp32_vs_fp64"] = {"steps": args.batch_err_steps, "rho": er[0], "U": er[1],
                                "T": er[2], "q_rel_to_max": er[3], "instances": len(sets)}
    # plain FP64 GPU path, one handle per instance, looped
    sample = sets[:: max(1, len(sets) // args.loop_sample)][: args.loop_sample]
    hs = []
    for KS in sample:
        ctr, face = kitgpu.init_fvm(KS, "fp64")
        hs.append((ctr.handle, kitgpu.timestep(KS, ctr, 0.0), KS.ps.nx * KS.vs.nu))
    for h, dt, _ in hs:
        h.step(dt, 2)
    t0 = time.perf_counter()
    for h, dt, _ in hs:
        h.step(dt, args.loop_steps)
    el = time.perf_counter() - t0
    for h, _, _ in hs:
        h.close()
    out["fp64_loop"] = {"value": sum(c for _, _, c in hs) * args.loop_steps / el, "unit": UNIT,
                        "instances_sampled": len(hs)}
    out["speedup_fp32_batch_vs_fp64_loop"] = out["fp32"]["value"] / out["fp64_loop"]["value"]
    return out


def unstruct_block(args, peak):
    """Unstructured 2D2F2V on a triangle mesh (a jittered triangulation of the
    unit square, n x n quads split in two), the reference's unstructured
    velocity grid and gas (test/t1_2f.txt: 16 x 16 velocities on [-5, 5]^2,
    Kn 0.075, Pr 1, inK 1, KFVS, BGK, first order) with extrapolated boundary
    cells, from a seeded smooth state.  FP32 split and plain FP64 step rates
    (CUDA events on the solve's stream), the step's HBM roofline fraction,
    end to end through the C ABI, the FP32 L-inf against FP64 after the same
    steps, and the oracle's CPU rate on a small mesh."""
    import torch
    from kitgpu import tune
    from kitgpu import unstruct as US
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    n = args.us_n
    P, T = US.rectangle_mesh(n, n, jitter=0.2, seed=11)
    m = US.build_mesh(P, T, boundary="extra")

    def prim_at(x, y):
        r2 = (x - 0.4) ** 2 + (y - 0.6) ** 2
        return np.array([1.0 + 0.4 * np.exp(-r2 / 0.03), 0.2 * np.sin(3 * y), -0.1 * np.cos(2 * x),
                         1.0 / (1.0 + 0.3 * np.exp(-r2 / 0.05))])

    KS = US.unstruct_solver_set(m, prim_at=prim_at)
    init = US.initial_cells(KS)
    nvel = KS.vs.nu * KS.vs.nv
    nstep_cells = int((m.cell_type == 0).sum())
    cv = m.ncell * nvel
    out = {"workload": "unstructured 2D2F2V, %d triangles (%dx%d jittered quads), %d stepped; "
                       "16x16 velocities on [-5,5]^2, KFVS + BGK, Kn=0.075, first order, "
                       "extrapolated boundary cells" % (m.ncell, n, n, nstep_cells),
           "cells": m.ncell, "velocities": nvel, "cell_velocity_per_step": cv}
    for prec, K in (("fp32", max(args.steps, 50)), ("fp64", max(2, min(args.steps, 10)))):
        hd = US.init_fvm(KS, prec)
        dt = hd.timestep()
        # stepped cells per CTA from the project autotuner (advances the
        # state, which is re-uploaded before timing)
        best, tim = tune.autotune_unstruct(hd, dt, steps=10, use_cache=not args.retune)
        hd.upload(*init)
        hd.step(dt, args.warmup)
        stream = torch.cuda.ExternalStream(hd.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n0 = hd.launches()
        torch.cuda.synchronize()
        e0.record(stream)
        hd.step(dt, K)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / K
        esz = 4 if prec == "fp32" else 8
        alg = 4.0 * esz * nstep_cells * nvel  # read h, b + write h, b of the stepped cells
        ach = alg / (ms / 1e3) / 1e9
        r = {"value": cv / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "steps": K,
             "gpu_launches": hd.launches() - n0, "cells_per_cta": hd.tuning(),
             "tuning_ms_per_step": tim,
             "roofline": {"bound": "hbm", "kernel": "k_us_step (whole step: k_us_step + boundary means)",
                          "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                          "algorithmic_bytes_per_step": alg}}
        # end to end: host FP64 state in, K steps, state out through the C ABI
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        hd.upload(*init)
        hd.step(dt, K)
        hd.download()
        el = time.perf_counter() - t0
        nb = sum(a.nbytes for a in init)
        r["e2e"] = {"value": cv * K / el, "unit": UNIT, "h2d_bytes_per_step": nb / K,
                    "d2h_bytes_per_step": nb / K}
        hd.close()
        out[prec] = r
    # FP32 against FP64 after the same number of steps
    Ke = 20
    st = {}
    for prec in ("fp32", "fp64"):
        hd = US.init_fvm(KS, prec)
        dt = hd.timestep()
        hd.step(dt, Ke)
        st[prec] = hd.download()
        hd.close()
    e = prim_errors(st["fp32"]["prim"], st["fp64"]["prim"])
    out["linf_fp32_vs_fp64"] = {"steps": Ke, "rho": e[0], "U": e[1], "T": e[2]}
    out["speedup_fp32_vs_fp64"] = out["fp32"]["value"] / out["fp64"]["value"]
    # the oracle (its C restatement, all host threads) on a 96 x 96-quad mesh
    if not args.no_cpu:
        import oracle_us as OU
        Ps, Ts = US.rectangle_mesh(96, 96, jitter=0.2, seed=11)
        ms_ = US.build_mesh(Ps, Ts, boundary="extra")
        KSs = US.unstruct_solver_set(ms_, prim_at=prim_at)
        vs, gs = KSs.vs, KSs.gas
        orc = OU.UnstructOracle(Ps, Ts, ms_.cell_type, vs.flat(vs.u), vs.flat(vs.v), vs.flat(vs.weights),
                                gs.K, gs.gamma, gs.mu_ref, gs.omega, gs.Pr, "bgk")
        orc.set_state(*US.initial_cells(KSs))
        orc.use_c()
        dt = orc.timestep(KSs.set.cfl, 0.0, KSs.set.maxTime, vs.u1, vs.v1)
        orc.step(dt, 2)
        t0 = time.perf_counter()
        ks = 0
        while time.perf_counter() - t0 < 10.0:
            orc.step(dt, 5)
            ks += 5
        el = time.perf_counter() - t0
        thr = os.cpu_count() or 1
        out["cpu_baseline"] = {"value": ms_.ncell * nvel * ks / el, "unit": UNIT, "cores": thr,
                               "kind": "port", "sample": "%d steps of the FP64 C oracle (OpenMP) on %d triangles"
                                                         % (ks, ms_.ncell)}
    return out


def run_unstruct(args):
    import torch
    torch.cuda.set_device(0)
    import kitgpu
    kitgpu.load()
    out = unstruct_block(args, measured_peaks()[0])
    print(json.dumps({"metric": METRIC, "workload": "unstructured", "result": out}), flush=True)
    return 0


def run_batch(args):
    import torch
    import kitgpu
    torch.cuda.set_device(0)
    kitgpu.load()
    out = batch_block(args, measured_peaks()[0])
    print(json.dumps({"metric": METRIC, "workload": "batch", "result": out}), flush=True)
    return 0


def serve_block(args):
    """Served mixed stream (Poisson arrivals): the FP32-split server at each
    offered rate with a realistic step cap, and the plain FP64 server against
    the FP32 one on one shorter stream (the FP64 form is ~100x slower)."""
    from kitgpu import serve as S
    mix = ("60% 1D Sod (cells 64..2048, velocities 32..256), 40% 2D cavity (16^2..128^2 cells, "
           "16^2..48^2 velocities, Kn 1e-4..1)")
    out = {"stream": {"mix": mix, "tol": 1e-6, "max_steps": args.max_steps,
                      "duration_s": args.duration}, "fp32": {}}
    for rate in args.rates:
        reqs = S.mixed_stream(rate=rate, duration=args.duration, seed=20261203,
                              max_steps=args.max_steps, tol=1e-6)
        srv = S.Server(precision="fp32", hbm_budget=args.hbm_gb << 30, max_slots=args.slots,
                       chunk=args.chunk)
        out["fp32"]["rate_%g" % rate] = srv.run(reqs)
    cmp_ = {"rate_per_s": 50.0, "duration_s": args.cmp_duration, "max_steps": args.cmp_steps}
    for prec in ("fp32", "fp64"):
        reqs = S.mixed_stream(rate=50.0, duration=args.cmp_duration, seed=20261203,
                              max_steps=args.cmp_steps, tol=1e-6)
        srv = S.Server(precision=prec, hbm_budget=args.hbm_gb << 30, max_slots=args.slots,
                       chunk=args.chunk)
        cmp_[prec] = srv.run(reqs)
    cmp_["throughput_ratio_fp32_vs_fp64"] = cmp_["fp32"]["throughput"] / cmp_["fp64"]["throughput"]
    out["same_stream_fp32_vs_fp64"] = cmp_
    return out


def run_serve(args):
    import torch
    import kitgpu
    torch.cuda.set_device(0)
    kitgpu.load()
    res = serve_block(args)
    print(json.dumps({"metric": METRIC + " and p50/p99 latency", "workload": "serve",
                      "result": res}), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--small", action="store_true", help="128x128 cells instead of 512x512")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-error", action="store_true")
    ap.add_argument("--err-steps", type=int, default=40)
    ap.add_argument("--retune", action="store_true", help="ignore the autotuner cache")
    ap.add_argument("--workload", choices=("quadrant", "batch", "serve", "unstructured"),
                    default="quadrant")
    ap.add_argument("--us-n", type=int, default=384, help="unstructured mesh: n x n quads, 2 n^2 triangles")
    ap.add_argument("--no-unstruct", action="store_true")
    ap.add_argument("--instances", type=int, default=512)
    ap.add_argument("--max-steady", type=int, default=40000)
    ap.add_argument("--loop-sample", type=int, default=64)
    ap.add_argument("--loop-steps", type=int, default=20)
    ap.add_argument("--batch-err-steps", type=int, default=400)
    ap.add_argument("--steady-sample", type=int, default=32)
    ap.add_argument("--steady-cap", type=int, default=10000)
    ap.add_argument("--rates", type=float, nargs="+", default=[20.0, 50.0, 200.0])
    ap.add_argument("--duration", type=float, default=2.0)
    ap.add_argument("--max-steps", type=int, default=2000)
    ap.add_argument("--cmp-duration", type=float, default=1.0)
    ap.add_argument("--cmp-steps", type=int, default=100)
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--slots", type=int, default=64)
    ap.add_argument("--chunk", type=int, default=20)
    ap.add_argument("--hbm-gb", type=int, default=64)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "serve":
        return run_serve(args)
    if args.workload == "unstructured":
        return run_unstruct(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
