"""Pick the fastest plan configuration for one geometry by measuring it.

The choices are those that change how the matrix is streamed, not what is
computed: slices per pass (K), the forward projection's scheduling
(ray-ordered gathers vs. 64x64 shared-memory reconstruction tiles) and the
backprojection's (L1 gathers vs. shared-memory detector windows). Each
candidate plan is built on a sample of the slices and timed over a few
iterations (host clock around synchronised calls); the fastest per
slice-iteration wins.
"""
from __future__ import annotations

import itertools
import time

from . import Plan, default_params

DEFAULT_SPACE = {
    "slices_per_pass": (4, 8),
    "forward_tiles": (False, True),
    "backward_staged": (False, True),
}


def autotune(theta, sino, alg="pml", params=None, *, len_storage="u16",
             space=None, iters=2, warmup=1, stream=None, log=None):
    """Time every configuration of `space` on `sino` ([P][S][C], host array or
    device tensor; S is the sample) and return (best, results).

    best: dict of Plan keyword arguments; results: list of
    (config, ms per slice-iteration, plan setup ms).
    """
    space = space or DEFAULT_SPACE
    P, S, C = (int(x) for x in sino.shape)
    params = params or default_params(alg)
    keys = list(space)
    results = []
    for values in itertools.product(*(space[k] for k in keys)):
        cfg = dict(zip(keys, values))
        t0 = time.perf_counter()
        plan = Plan(P, S, C, theta, len_storage=len_storage, mode="fast",
                    delta_index=True, **cfg)
        if stream is not None:
            plan.set_stream(stream)
        setup_ms = (time.perf_counter() - t0) * 1e3
        plan.set_sinogram(sino, apply_abs=alg != "sirt")
        plan.reset_recon(alg)
        plan.iterate(alg, warmup, params)
        plan.synchronize()
        t1 = time.perf_counter()
        plan.iterate(alg, iters, params)
        plan.synchronize()
        ms = (time.perf_counter() - t1) * 1e3 / (iters * S)
        results.append((cfg, ms, setup_ms))
        if log:
            log(f"autotune {cfg}: {ms:.3f} ms per slice-iteration")
        plan.close()
    best = min(results, key=lambda r: r[1])[0]
    return dict(best), results
