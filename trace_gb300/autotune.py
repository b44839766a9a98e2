"""Pick the fastest plan configuration for one geometry by measuring it.

The choices are those that change how the system matrix is held and
streamed, not what is computed: slices per pass (K), the forward
projection's scheduling (ray-ordered gathers vs. shared-memory
reconstruction tiles, the tiles' side and the warps - runs in flight - of
each tile's block), the backprojection's (L1 gathers
vs. shared-memory detector windows, and the pixel-tile shape a warp covers),
and cached vs. on-the-fly ray intersections for the ray-ordered forward
projection. Each candidate plan is built on a sample of the slices and timed
over a few iterations (host clock around synchronised calls); the fastest
per slice-iteration wins. With a device-memory budget, configurations whose
plan needs more are skipped, which is where tracing on the fly (no stored
forward matrix) earns its place.

The search is the full product of DEFAULT_SPACE (schedule choices that
interact), then one dimension of REFINE_SPACE at a time from the best so far
(tile side and tile shape are independent refinements of the kernels the
schedule picked).
"""
from __future__ import annotations

import itertools
import math
import time

from . import Plan, TraceError, default_params

DEFAULT_SPACE = {
    "slices_per_pass": (4, 8, 16),
    "forward_tiles": (False, True),
    "backward_staged": (False, True),
    "forward_on_the_fly": (False, True),
}

# refined one at a time from the best configuration of DEFAULT_SPACE
REFINE_SPACE = {
    "forward_tile_side": (32, 48, 64, 80, 96),  # forward_tiles: shared-memory tile side
    "backward_tile_width": (4, 8, 16),     # backprojection tiles 4x8, 8x4, 16x2
    "forward_block_warps": (8, 16, 32),    # forward_tiles: runs in flight per tile
}
# what a plan uses when the key is not given
PLAN_DEFAULTS = {"forward_tile_side": 64, "backward_tile_width": 8, "forward_block_warps": 32}

TG_E_ARG = 1
TG_E_NOMEM = 3


def _measure(theta, sino, alg, params, len_storage, cfg, fixed, iters, warmup, stream,
             max_device_bytes):
    """(ms per slice-iteration, setup ms, device bytes) of one configuration;
    None if the plan rejects the combination."""
    P, S, C = (int(x) for x in sino.shape)
    t0 = time.perf_counter()
    try:
        plan = Plan(P, S, C, theta, len_storage=len_storage, mode="fast",
                    delta_index=True, **{**(fixed or {}), **cfg})
    except TraceError as e:
        if e.status == TG_E_ARG:
            return None  # not a valid combination (e.g. half_gathers + staged)
        if e.status != TG_E_NOMEM:
            raise
        return math.inf, 0.0, None
    setup_ms = (time.perf_counter() - t0) * 1e3
    nbytes = plan.info()["device_bytes"]
    if max_device_bytes is not None and nbytes > max_device_bytes:
        plan.close()
        return math.inf, setup_ms, nbytes
    if stream is not None:
        plan.set_stream(stream)
    plan.set_sinogram(sino, apply_abs=alg != "sirt")
    plan.reset_recon(alg)
    plan.iterate(alg, warmup, params)
    plan.synchronize()
    t1 = time.perf_counter()
    plan.iterate(alg, iters, params)
    plan.synchronize()
    ms = (time.perf_counter() - t1) * 1e3 / (iters * S)
    plan.close()
    return ms, setup_ms, nbytes


def autotune(theta, sino, alg="pml", params=None, *, len_storage="u16",
             space=None, refine=None, iters=2, warmup=1, stream=None, log=None,
             max_device_bytes=None, fixed=None):
    """Time the configurations of `space` (full product) and then of `refine`
    (one dimension at a time) on `sino` ([P][S][C], host array or device
    tensor; S is the sample) and return (best, results).

    best: dict of Plan keyword arguments; results: list of
    (config, ms per slice-iteration, plan setup ms, plan device bytes), with
    ms = inf for configurations that did not fit `max_device_bytes` (or the
    device). `fixed`: Plan keyword arguments held for every candidate (e.g.
    half_gathers); combinations a plan rejects as invalid are skipped.
    refine=None uses REFINE_SPACE; pass {} to skip the refinement.
    """
    space = space or DEFAULT_SPACE
    refine = REFINE_SPACE if refine is None else refine
    params = params or default_params(alg)
    results = []

    def run(cfg):
        r = _measure(theta, sino, alg, params, len_storage, cfg, fixed, iters, warmup,
                     stream, max_device_bytes)
        if r is None:
            return None
        results.append((dict(cfg), *r))
        if log:
            log(f"autotune {cfg}: {r[0]:.3f} ms per slice-iteration")
        return r[0]

    keys = list(space)
    for values in itertools.product(*(space[k] for k in keys)):
        cfg = dict(zip(keys, values))
        if (cfg.get("forward_on_the_fly") and cfg.get("forward_tiles")
                and max_device_bytes is None):
            continue  # iterations use the tiles either way; only memory differs
        run(cfg)
    fitting = [r for r in results if math.isfinite(r[1])]
    if not fitting:
        raise RuntimeError("no configuration fits the device-memory budget")
    best_cfg, best_ms = min(fitting, key=lambda r: r[1])[:2]
    best_cfg = dict(best_cfg)
    for key, values in refine.items():
        if key in ("forward_tile_side", "forward_block_warps") and not best_cfg.get(
                "forward_tiles"):
            continue
        for v in values:
            if key not in best_cfg and v == PLAN_DEFAULTS.get(key):
                continue  # the configuration already measured
            cfg = {**best_cfg, key: v}
            if any(c == cfg for c, *_ in results):
                continue
            ms = run(cfg)
            if ms is not None and ms < best_ms:
                best_cfg, best_ms = cfg, ms
    return best_cfg, results
