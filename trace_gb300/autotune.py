"""Pick the fastest plan configuration for one geometry by measuring it.

The choices are those that change how the system matrix is held and
streamed, not what is computed: slices per pass (K), the forward
projection's scheduling (ray-ordered gathers vs. 64x64 shared-memory
reconstruction tiles), the backprojection's (L1 gathers vs. shared-memory
detector windows), and cached vs. on-the-fly ray intersections for the
ray-ordered forward projection. Each candidate plan is built on a sample of
the slices and timed over a few iterations (host clock around synchronised
calls); the fastest per slice-iteration wins. With a device-memory budget,
configurations whose plan needs more are skipped, which is where tracing on
the fly (no stored forward matrix) earns its place.
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

TG_E_ARG = 1
TG_E_NOMEM = 3


def autotune(theta, sino, alg="pml", params=None, *, len_storage="u16",
             space=None, iters=2, warmup=1, stream=None, log=None,
             max_device_bytes=None, fixed=None):
    """Time every configuration of `space` on `sino` ([P][S][C], host array or
    device tensor; S is the sample) and return (best, results).

    best: dict of Plan keyword arguments; results: list of
    (config, ms per slice-iteration, plan setup ms, plan device bytes), with
    ms = inf for configurations that did not fit `max_device_bytes` (or the
    device). `fixed`: Plan keyword arguments held for every candidate (e.g.
    half_gathers); combinations a plan rejects as invalid are skipped.
    """
    space = space or DEFAULT_SPACE
    P, S, C = (int(x) for x in sino.shape)
    params = params or default_params(alg)
    keys = list(space)
    results = []
    for values in itertools.product(*(space[k] for k in keys)):
        cfg = dict(zip(keys, values))
        if (cfg.get("forward_on_the_fly") and cfg.get("forward_tiles")
                and max_device_bytes is None):
            continue  # iterations use the tiles either way; only memory differs
        t0 = time.perf_counter()
        try:
            plan = Plan(P, S, C, theta, len_storage=len_storage, mode="fast",
                        delta_index=True, **{**(fixed or {}), **cfg})
        except TraceError as e:
            if e.status == TG_E_ARG:
                continue  # not a valid combination (e.g. half_gathers + staged)
            if e.status != TG_E_NOMEM:
                raise
            results.append((cfg, math.inf, 0.0, None))
            continue
        setup_ms = (time.perf_counter() - t0) * 1e3
        nbytes = plan.info()["device_bytes"]
        if max_device_bytes is not None and nbytes > max_device_bytes:
            plan.close()
            results.append((cfg, math.inf, setup_ms, nbytes))
            continue
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
        results.append((cfg, ms, setup_ms, nbytes))
        if log:
            log(f"autotune {cfg}: {ms:.3f} ms per slice-iteration, {nbytes / 1e9:.2f} GB")
        plan.close()
    fitting = [r for r in results if math.isfinite(r[1])]
    if not fitting:
        raise RuntimeError("no configuration fits the device-memory budget")
    best = min(fitting, key=lambda r: r[1])[0]
    return dict(best), results
