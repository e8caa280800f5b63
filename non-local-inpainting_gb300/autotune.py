"""Autotuner for the launch shapes the library leaves open: the size of the
thread-block clusters of the NL-Poisson conjugate gradient (CTAs per
cluster, unknowns per CTA), the largest CG system one CTA solves alone
(NLI_TUNE_CG_SINGLE_MAX), the way the 9x9 PatchMatch kernels read their
windows (NLI_TUNE_PM_VARIANT), the PatchMatch lower-bound test
(NLI_TUNE_PM_BOUND) and work distribution (NLI_TUNE_PM_TILE: static ranges
or a device work queue, and its tile), how a batch runs (NLI_TUNE_BATCH_MODE, the worker
contexts' width, the lockstep sub-groups NLI_TUNE_BATCH_GROUPS).  Each
candidate is timed with CUDA events on a representative case on the
context's own device; the fastest is set on the context
(nli_ctx_set_tuning) and returned with the whole table, which callers may
store and re-apply with apply().  Results depend on these shapes only
through the float rounding of the CG's sums; the PatchMatch variants and
the bound give identical fields, the batch forms identical images.
"""
from __future__ import annotations

import itertools


def _events(torch):
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def poisson_case(ctx, size=512, hole=0.15, seed=0):
    """A finest-level NL-Poisson update case: Voronoi texture, ellipse hole,
    NNF from a seeded PatchMatch call, confidence of the hole."""
    import numpy as np
    from . import workloads as wl
    rng = np.random.default_rng(seed)
    img, _ = wl.voronoi_texture(size, size, 40, rng)
    mask = wl.ellipse_mask(size, size, 6, hole, rng)
    p = wl.params("nlpoisson", scales=2, coarse=0.5, iters=1, cg_tol=1e-4)
    ext = ctx.extended_domain(mask, 9, 9)
    src, tgt, _ = ctx.scale_masks(ext, 4, True)
    u = ctx.poisson_init(img, mask)
    ctx.set_seed(seed)
    nnf, _, _ = ctx.patchmatch(p.distance, p.patchmatch, u, src, u, tgt)
    conf = ctx.confidence_mask(mask, 5.0, 0.1)
    return p.update, u, mask, ext, nnf, conf


def tune_cg(ctx, case=None, caps=(4, 8, 12, 16), per_cta=(512, 1024, 2048), repeats=3):
    """Times one NL-Poisson update per (cluster cap, unknowns per CTA) and
    keeps the fastest.  Returns {"best": (cap, per), "ms": {(cap, per): ms}}."""
    import torch
    upd, u, mask, ext, nnf, conf = case if case is not None else poisson_case(ctx)
    times = {}
    for cap, per in itertools.product(caps, per_cta):
        ctx.set_tuning(ctx.TUNE_CG_CLUSTER_CAP, cap)
        ctx.set_tuning(ctx.TUNE_CG_UNKNOWNS_PER_CTA, per)
        ctx.update(upd, u, u, mask, ext, nnf, conf)  # warm
        best = float("inf")
        for _ in range(repeats):
            torch.cuda.synchronize()
            a, b = _events(torch)
            a.record()
            ctx.update(upd, u, u, mask, ext, nnf, conf)
            b.record()
            torch.cuda.synchronize()
            best = min(best, a.elapsed_time(b))
        times[(cap, per)] = best
    choice = min(times, key=times.get)
    ctx.set_tuning(ctx.TUNE_CG_CLUSTER_CAP, choice[0])
    ctx.set_tuning(ctx.TUNE_CG_UNKNOWNS_PER_CTA, choice[1])
    return {"best": choice, "ms": times}


def patchmatch_case(ctx, size=512, hole=0.15, seed=0):
    """A finest-level PatchMatch case (9x9 L2 combined, 10 sweeps): Poisson
    filled Voronoi texture with an ellipse hole and the driver's masks."""
    import numpy as np
    from . import workloads as wl
    rng = np.random.default_rng(seed)
    img, _ = wl.voronoi_texture(size, size, 40, rng)
    mask = wl.ellipse_mask(size, size, 6, hole, rng)
    p = wl.params("nlpoisson", scales=2, coarse=0.5, iters=1, cg_tol=1e-4)
    ext = ctx.extended_domain(mask, 9, 9)
    src, tgt, _ = ctx.scale_masks(ext, 4, True)
    u = ctx.poisson_init(img, mask)
    return p.distance, p.patchmatch, u, src, tgt


def tune_pm_variant(ctx, case=None, variants=(0, 1, 2), repeats=3, seed=0):
    """Times one PatchMatch call per window variant and keeps the fastest.
    Returns {"best": variant, "ms": {variant: ms}}."""
    import torch
    dist, pm, u, src, tgt = case if case is not None else patchmatch_case(ctx)
    times = {}
    for v in variants:
        ctx.set_tuning(ctx.TUNE_PM_VARIANT, v)
        ctx.set_seed(seed)
        ctx.patchmatch(dist, pm, u, src, u, tgt, want_energy=False)  # warm
        best = float("inf")
        for _ in range(repeats):
            ctx.set_seed(seed)
            torch.cuda.synchronize()
            a, b = _events(torch)
            a.record()
            ctx.patchmatch(dist, pm, u, src, u, tgt, want_energy=False)
            b.record()
            torch.cuda.synchronize()
            best = min(best, a.elapsed_time(b))
        times[v] = best
    choice = min(times, key=times.get)
    ctx.set_tuning(ctx.TUNE_PM_VARIANT, choice)
    return {"best": choice, "ms": times}


def tune_batch_width(ctx, items, params, widths=(2, 4, 8, 12, 16)):
    """Times process_batch_device on device-resident `items` per batch width
    and keeps the fastest.  Returns {"best": width, "ms": {width: ms}}."""
    import torch
    times = {}
    for w in widths:
        ctx.set_batch_width(w)
        torch.cuda.synchronize()
        a, b = _events(torch)
        a.record()
        ctx.process_batch_device(items, params)
        b.record()
        torch.cuda.synchronize()
        times[w] = a.elapsed_time(b)
    choice = min(times, key=times.get)
    ctx.set_batch_width(choice)
    return {"best": choice, "ms": times}


def _time_update(ctx, case, repeats):
    import torch
    upd, u, mask, ext, nnf, conf = case
    ctx.update(upd, u, u, mask, ext, nnf, conf)  # warm
    best = float("inf")
    for _ in range(repeats):
        torch.cuda.synchronize()
        a, b = _events(torch)
        a.record()
        ctx.update(upd, u, u, mask, ext, nnf, conf)
        b.record()
        torch.cuda.synchronize()
        best = min(best, a.elapsed_time(b))
    return best


def tune_cg_single(ctx, cases=None, limits=(0, 512, 1024, 2048, 4096), repeats=3):
    """Times NL-Poisson updates of a few small systems (the coarse pyramid
    levels' sizes) per one-CTA limit and keeps the limit with the smallest
    total.  Returns {"best": limit, "ms": {limit: ms}}."""
    if cases is None:
        cases = [poisson_case(ctx, size=s, seed=1) for s in (48, 72, 96, 128)]
    times = {}
    for lim in limits:
        ctx.set_tuning(ctx.TUNE_CG_SINGLE_MAX, lim)
        times[lim] = sum(_time_update(ctx, c, repeats) for c in cases)
    choice = min(times, key=times.get)
    ctx.set_tuning(ctx.TUNE_CG_SINGLE_MAX, choice)
    return {"best": choice, "ms": times}


def tune_pm_bound(ctx, case=None, repeats=3, seed=0):
    """Times one PatchMatch call per lower-bound mode (0 none, 1 patch
    means, 2 means and deviations) and keeps the fastest.  Returns
    {"best": mode, "ms": {mode: ms}}."""
    import torch
    dist, pm, u, src, tgt = case if case is not None else patchmatch_case(ctx)
    times = {}
    for v in (0, 1, 2):
        ctx.set_tuning(ctx.TUNE_PM_BOUND, v)
        ctx.set_seed(seed)
        ctx.patchmatch(dist, pm, u, src, u, tgt, want_energy=False)  # warm
        best = float("inf")
        for _ in range(repeats):
            ctx.set_seed(seed)
            torch.cuda.synchronize()
            a, b = _events(torch)
            a.record()
            ctx.patchmatch(dist, pm, u, src, u, tgt, want_energy=False)
            b.record()
            torch.cuda.synchronize()
            best = min(best, a.elapsed_time(b))
        times[v] = best
    choice = min(times, key=times.get)
    ctx.set_tuning(ctx.TUNE_PM_BOUND, choice)
    return {"best": choice, "ms": times}


def tune_pm_tile(ctx, case=None, tiles=(0, 4, 16, 64), repeats=3, seed=0):
    """Times one PatchMatch call per work distribution (0: static block
    ranges; n: a device work queue handing out n target points per grab)
    and keeps the fastest.  Returns {"best": tile, "ms": {tile: ms}}."""
    import torch
    dist, pm, u, src, tgt = case if case is not None else patchmatch_case(ctx)
    times = {}
    for v in tiles:
        ctx.set_tuning(ctx.TUNE_PM_TILE, v)
        ctx.set_seed(seed)
        ctx.patchmatch(dist, pm, u, src, u, tgt, want_energy=False)  # warm
        best = float("inf")
        for _ in range(repeats):
            ctx.set_seed(seed)
            torch.cuda.synchronize()
            a, b = _events(torch)
            a.record()
            ctx.patchmatch(dist, pm, u, src, u, tgt, want_energy=False)
            b.record()
            torch.cuda.synchronize()
            best = min(best, a.elapsed_time(b))
        times[v] = best
    choice = min(times, key=times.get)
    ctx.set_tuning(ctx.TUNE_PM_TILE, choice)
    return {"best": choice, "ms": times}


def _time_batch(ctx, items, params):
    import torch
    torch.cuda.synchronize()
    a, b = _events(torch)
    a.record()
    ctx.process_batch_device(items, params)
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b)


def tune_batch_mode(ctx, items, params):
    """Times process_batch_device on device-resident `items` in the lockstep
    form (1) and the worker-context form (0) and keeps the faster.  Returns
    {"best": mode, "ms": {mode: ms}}."""
    times = {}
    for mode in (1, 0):
        ctx.set_tuning(ctx.TUNE_BATCH_MODE, mode)
        times[mode] = _time_batch(ctx, items, params)
    choice = min(times, key=times.get)
    ctx.set_tuning(ctx.TUNE_BATCH_MODE, choice)
    return {"best": choice, "ms": times}


def tune_batch_groups(ctx, items, params, groups=(1, 2, 4)):
    """Times lockstep process_batch_device on device-resident `items` per
    number of concurrent sub-groups and keeps the fastest.  Returns
    {"best": groups, "ms": {groups: ms}}."""
    mode = ctx.get_tuning(ctx.TUNE_BATCH_MODE)
    ctx.set_tuning(ctx.TUNE_BATCH_MODE, 1)
    times = {}
    try:
        for g in groups:
            ctx.set_tuning(ctx.TUNE_BATCH_GROUPS, g)
            times[g] = _time_batch(ctx, items, params)
    finally:
        ctx.set_tuning(ctx.TUNE_BATCH_MODE, mode)
    choice = min(times, key=times.get)
    ctx.set_tuning(ctx.TUNE_BATCH_GROUPS, choice)
    return {"best": choice, "ms": times}


def device_key(device=0):
    """The cache key of a device: its name, SM count and compute capability."""
    import torch
    pr = torch.cuda.get_device_properties(device)
    return "%s|%d SMs|sm_%d%d" % (pr.name, pr.multi_processor_count, pr.major, pr.minor)


_SCALARS = ("batch_width", "pm_variant", "cg_single", "pm_bound", "batch_mode", "batch_groups", "pm_tile")


def save(path, key, cg=None, batch_width=None, pm_variant=None, cg_single=None, pm_bound=None, batch_mode=None,
         batch_groups=None, pm_tile=None):
    """Stores the choices for one device key in a JSON cache file (other
    devices' entries are kept)."""
    import json
    import os
    table = {}
    if os.path.exists(path):
        with open(path) as f:
            table = json.load(f)
    entry = {}
    if cg is not None:
        entry["cg"] = [int(cg[0]), int(cg[1])]
    values = dict(batch_width=batch_width, pm_variant=pm_variant, cg_single=cg_single, pm_bound=pm_bound,
                  batch_mode=batch_mode, batch_groups=batch_groups, pm_tile=pm_tile)
    for name in _SCALARS:
        if values[name] is not None:
            entry[name] = int(values[name])
    table[key] = entry
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def load(ctx, path, key):
    """Applies the cached choices of `key` to ctx; returns them, or None
    when the file or the key is absent."""
    import json
    import os
    if not os.path.exists(path):
        return None
    with open(path) as f:
        entry = json.load(f).get(key)
    if entry is None:
        return None
    apply(ctx, cg=entry.get("cg"), **{name: entry.get(name) for name in _SCALARS})
    return entry


def apply(ctx, cg=None, batch_width=None, pm_variant=None, cg_single=None, pm_bound=None, batch_mode=None,
          batch_groups=None, pm_tile=None):
    """Re-applies stored choices: cg = (cap, unknowns per CTA)."""
    if cg is not None:
        ctx.set_tuning(ctx.TUNE_CG_CLUSTER_CAP, int(cg[0]))
        ctx.set_tuning(ctx.TUNE_CG_UNKNOWNS_PER_CTA, int(cg[1]))
    for knob, value in ((ctx.TUNE_PM_VARIANT, pm_variant), (ctx.TUNE_CG_SINGLE_MAX, cg_single),
                        (ctx.TUNE_PM_BOUND, pm_bound), (ctx.TUNE_BATCH_MODE, batch_mode),
                        (ctx.TUNE_BATCH_GROUPS, batch_groups), (ctx.TUNE_PM_TILE, pm_tile)):
        if value is not None:
            ctx.set_tuning(knob, int(value))
    if batch_width is not None:
        ctx.set_batch_width(int(batch_width))
