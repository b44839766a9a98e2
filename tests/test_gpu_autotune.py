"""The autotuner (trace_gb300.autotune): times the schedule choices on a
sample and returns a configuration a plan accepts; under a device-memory
budget it keeps to configurations that fit (tracing on the fly when only
that fits)."""
import math

import numpy as np
import pytest

import trace_gb300 as tg
from trace_gb300.autotune import autotune
from tests._util import ellipse_sino, rel_l2

pytestmark = pytest.mark.gpu


def test_autotune_returns_a_working_configuration():
    C, P, S = 96, 72, 8
    th, tabs, _, sino = ellipse_sino(C, P, S, seed=3)
    best, res = autotune(th, sino, "mlem", iters=1, warmup=1)
    assert any(r[0] == best and math.isfinite(r[1]) for r in res)
    plan = tg.Plan(P, S, C, th, len_storage="u16", mode="fast", delta_index=True, **best)
    plan.set_sinogram(sino, apply_abs=True)
    plan.reset_recon("mlem")
    plan.iterate("mlem", 2)
    assert np.isfinite(plan.get_recon("mlem")).all()
    plan.close()


def test_autotune_budget_selects_on_the_fly_tracing():
    C, P, S = 96, 72, 4
    th, tabs, _, sino = ellipse_sino(C, P, S, seed=4)
    kw = dict(len_storage="u16", mode="fast", delta_index=True, slices_per_pass=4)
    sizes = {}
    for otf in (False, True):
        p = tg.Plan(P, S, C, th, forward_on_the_fly=otf, **kw)
        sizes[otf] = p.info()["device_bytes"]
        p.close()
    assert sizes[True] < sizes[False]
    space = {"slices_per_pass": (4,), "forward_tiles": (False, True),
             "backward_staged": (False,), "forward_on_the_fly": (False, True)}
    best, res = autotune(th, sino, "sirt", space=space, refine={}, iters=1, warmup=1,
                         max_device_bytes=sizes[True])
    assert best["forward_on_the_fly"] and not best["forward_tiles"]
    assert sum(math.isfinite(r[1]) for r in res) == 1


def test_autotune_refines_tile_side_and_tile_shape():
    """With the refinement dimensions the autotuner measures forward tile
    sides and backprojection tile shapes from the best schedule, and the
    configuration it returns is one it measured."""
    from tests._util import theta_uniform
    C, P, S = 128, 90, 8
    th = theta_uniform(P)
    rng = np.random.default_rng(3)
    sino = rng.uniform(0.5, 2.0, (P, S, C)).astype(np.float32)
    best, res = autotune(th, sino, "mlem", space={"slices_per_pass": (8,),
                                                   "forward_tiles": (True,)},
                         fixed={"half_gathers": True})
    cfgs = [c for c, *_ in res]
    assert any(c.get("forward_tile_side") == 32 for c in cfgs)
    assert any(c.get("backward_tile_width") in (4, 16) for c in cfgs)
    assert best in cfgs
    plan = tg.Plan(P, S, C, th, len_storage="u16", mode="fast", delta_index=True,
                   half_gathers=True, **best)
    plan.close()
