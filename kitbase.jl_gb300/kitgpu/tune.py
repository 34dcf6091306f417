"""Autotuner of the launch shapes of the two HBM passes.

For a handle it times candidate shapes of the pointwise update pass (columns
per strip, rows per CTA, threads per CTA) and of the moment pass (faces per
warp) with the library's own CUDA-event stage timing, on the handle's real
state, and keeps the fastest.  Results are cached per problem signature
(dimension, velocity count, flux, collision, precision, grid size class) in a
JSON file so repeated solves of the same shape skip the search.

The search advances the solution by a few steps; callers that need the
original state re-upload it (bench.py does) or tune on a copy.
"""
import itertools
import json
import os

from . import _native as N

CACHE = os.environ.get("KITGPU_TUNE_CACHE",
                       os.path.join(os.path.expanduser("~"), ".cache", "kitgpu_tune.json"))

MARCH_TX = (2, 4)
MARCH_BS = (64, 128)
MARCH_RY = (16, 32, 64)
MOM_TS = (2, 4, 8)  # faces per warp of the line form; 8: the row-ring form (2D FP32 BGK)


def signature(handle):
    c = handle.cfg
    cells = c.nx * (c.ny if c.dim == 2 else 1)
    size = "small" if cells < 4096 else ("medium" if cells < 65536 else "large")
    return "d%d-v%d-f%d-c%d-p%d-%s" % (c.dim, handle.nvel, c.flux, c.collision, c.precision, size)


def _load():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(d):
    try:
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        with open(CACHE, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
    except OSError:
        pass


def _time(handle, dt, steps):
    handle.set_timing(True)
    handle.step(dt, steps)
    t = handle.timing()
    handle.set_timing(False)
    upd = t["update"][0] / max(t["update"][1], 1)
    mom = t["moments"][0] / max(t["moments"][1], 1)
    return upd, mom


def autotune(handle, dt, steps=2, use_cache=True, verbose=False):
    """Pick the fastest launch shapes for `handle`; returns the chosen dict and
    the per-candidate timings (ms per step of each pass)."""
    key = signature(handle)
    cache = _load() if use_cache else {}
    if use_cache and key in cache:
        best = cache[key]
        handle.set_tuning(**best)
        return best, None
    res_march = {}
    ry_opts = MARCH_RY if handle.dim == 2 else (1,)
    for tx, bs, ry in itertools.product(MARCH_TX, MARCH_BS, ry_opts):
        handle.set_tuning(march_tx=tx, march_ry=ry, march_bs=bs, mom_ts=0)
        handle.step(dt, 1)  # warm-up of this shape
        upd, _ = _time(handle, dt, steps)
        res_march[(tx, bs, ry)] = upd
        if verbose:
            print("march tx=%d bs=%d ry=%d: %.3f ms" % (tx, bs, ry, upd), flush=True)
    tx, bs, ry = min(res_march, key=res_march.get)
    res_mom = {}
    for ts in MOM_TS:
        handle.set_tuning(march_tx=tx, march_ry=ry, march_bs=bs, mom_ts=ts)
        handle.step(dt, 1)
        _, mom = _time(handle, dt, steps)
        res_mom[ts] = mom
        if verbose:
            print("moments ts=%d: %.3f ms" % (ts, mom), flush=True)
    ts = min(res_mom, key=res_mom.get)
    best = dict(march_tx=tx, march_ry=ry, march_bs=bs, mom_ts=ts)
    handle.set_tuning(**best)
    if use_cache:
        cache[key] = best
        _save(cache)
    timings = {"march": {"tx%d-bs%d-ry%d" % k: v for k, v in res_march.items()},
               "moments": {"ts%d" % k: v for k, v in res_mom.items()}}
    return best, timings


# Shapes of the fused FP32 batch step kernel (kb_batch_set_tuning): cells per
# segment x threads per CTA, each with one CTA per segment or a persistent
# grid of as many CTAs as fit on the GPU.
BATCH_SHAPES = ((8, 64), (16, 64), (16, 128), (16, 256), (32, 128), (32, 256))
BATCH_PERSIST = (0, 1)


def batch_signature(batch):
    n = batch.n
    cv = batch.cell_velocity_points()
    size = "small" if cv < 1 << 20 else ("medium" if cv < 1 << 24 else "large")
    return "batch-n%d-nu%d-c%s-%s" % (n, int(batch.nu.max()), batch.KS[0].set.collision, size)


def autotune_batch(batch, steps=100, use_cache=True, verbose=False):
    """Pick the fastest shape of the FP32 batch step for `batch` by timing
    `steps` graph-replayed steps of each candidate on the live state
    (kb_batch_step returns after synchronising the batch's stream; the search
    advances the state).  Returns the chosen dict and the per-candidate ms
    per step."""
    import time
    if batch.prec != "fp32":
        return None, None
    key = batch_signature(batch)
    cache = _load() if use_cache else {}
    if use_cache and key in cache:
        best = cache[key]
        batch.set_tuning(**best)
        return best, None
    res = {}
    for (seg, thr), per in itertools.product(BATCH_SHAPES, BATCH_PERSIST):
        batch.set_tuning(seg=seg, threads=thr, persist=per)
        batch.step(4)  # graph capture of this shape, warm-up
        t0 = time.perf_counter()
        batch.step(steps)
        res[(seg, thr, per)] = 1e3 * (time.perf_counter() - t0) / steps
        if verbose:
            print("batch seg=%d threads=%d persist=%d: %.4f ms" % (seg, thr, per, res[(seg, thr, per)]),
                  flush=True)
    seg, thr, per = min(res, key=res.get)
    best = dict(seg=seg, threads=thr, persist=per)
    batch.set_tuning(**best)
    if use_cache:
        cache[key] = best
        _save(cache)
    return best, {"seg%d-t%d-p%d" % k: v for k, v in res.items()}


US_CELLS_PER_CTA = (4, 8, 12, 16, 24, 32)


def unstruct_signature(hd):
    size = "small" if hd.ncell < 4096 else ("medium" if hd.ncell < 65536 else "large")
    return "us-v%d-c%d-p%d-%s" % (hd.nvel, hd.cfg.collision, hd.cfg.precision, size)


def autotune_unstruct(hd, dt, steps=20, use_cache=True, verbose=False):
    """Pick the fastest stepped-cells-per-CTA shape of the unstructured step
    for handle `hd` (kitgpu.unstruct.UnstructHandle) by timing `steps` steps of
    each candidate on the live state (kb_us_step returns after synchronising
    the solve's stream; the search advances the state).  Returns the chosen
    count and the per-candidate ms per step."""
    import time
    key = unstruct_signature(hd)
    cache = _load() if use_cache else {}
    if use_cache and key in cache:
        best = cache[key]["cells_per_cta"]
        hd.set_tuning(best)
        return best, None
    res = {}
    for cb in US_CELLS_PER_CTA:
        try:
            hd.set_tuning(cb)
        except N.KitGPUError:
            continue  # more shared memory than a CTA may have
        hd.step(dt, 2)
        t0 = time.perf_counter()
        hd.step(dt, steps)
        res[cb] = 1e3 * (time.perf_counter() - t0) / steps
        if verbose:
            print("unstructured cells/CTA=%d: %.4f ms" % (cb, res[cb]), flush=True)
    best = min(res, key=res.get)
    hd.set_tuning(best)
    if use_cache:
        cache[key] = {"cells_per_cta": best}
        _save(cache)
    return best, {"cb%d" % k: v for k, v in res.items()}
