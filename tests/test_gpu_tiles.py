"""Tile-staged forward projection (fast mode, forward_tiles=1) against the
ray-ordered fast path and the FP64 oracle."""
import numpy as np
import pytest

import trace_gb300 as tg
from oracle import oracle as O
from tests._util import rel_l2, theta_uniform

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("C,P,S,K", [(100, 60, 5, 1), (128, 90, 4, 2), (130, 70, 6, 4),
                                     (96, 50, 9, 8)])
@pytest.mark.parametrize("alg", ["sirt", "mlem", "pml", "apmlr"])
@pytest.mark.parametrize("staged", [False, True])
def test_tiled_forward_matches_ray_ordered(C, P, S, K, alg, staged):
    th = theta_uniform(P)
    rng = np.random.default_rng(C + K)
    sino = rng.uniform(0.5, 2.0, (P, S, C)).astype(np.float32)
    prm = tg.default_params(alg, beta=0.2)
    outs = []
    for tiles in (False, True):
        plan = tg.Plan(P, S, C, th, slices_per_pass=K, mode="fast", len_storage="u16",
                       delta_index=True, forward_tiles=tiles,
                       backward_staged=staged and tiles)
        plan.set_sinogram(sino, apply_abs=alg != "sirt")
        plan.reset_recon(alg)
        plan.iterate(alg, 3, prm)
        outs.append(plan.get_recon(alg))
        if tiles:
            info = plan.info()
            assert info["tile_runs"] > 0 and info["tile_bytes"] > 0
        plan.close()
    assert rel_l2(outs[1], outs[0]) < 2e-6


@pytest.mark.parametrize("storage", ["f32", "f16", "bf16", "u16"])
def test_tiled_forward_storage_kinds_against_fp64(storage):
    C, P, S = 96, 72, 4
    th = theta_uniform(P)
    tabs = O.angle_table(th)
    from trace_gb300.phantom import ellipse_phantoms
    sino = O.forward(ellipse_phantoms(C, S, seed=3), tabs)
    ref = O.run("pml", sino, tables=tabs, n_iter=6, precision=O.F64, beta=0.05)["recon"]
    plan = tg.Plan(P, S, C, th, slices_per_pass=4, mode="fast", len_storage=storage,
                   delta_index=True, forward_tiles=True)
    plan.set_sinogram(sino, apply_abs=True)
    plan.reset_recon("pml")
    plan.iterate("pml", 6, tg.default_params("pml", beta=0.05))
    err = rel_l2(plan.get_recon("pml"), ref)
    assert err < (3e-3 if storage == "bf16" else 1e-4), err
    plan.close()


def test_forward_tiles_needs_fast_mode():
    with pytest.raises(tg.TraceError) as e:
        tg.Plan(8, 1, 16, theta_uniform(8), forward_tiles=True)
    assert e.value.status == 1
