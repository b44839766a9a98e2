"""Smallest and ragged geometries: two detector columns, one angle, one
slice; column counts off the 32-ray groups and the pixel tiles; slice
counts off the slices per pass. Exact mode against the oracle (the
reference's algorithm, float), fast tile-staged paths against FP64."""
import numpy as np
import pytest

import trace_gb300 as tg
from oracle import oracle as O
from tests._util import rel_l2, theta_uniform

pytestmark = pytest.mark.gpu

GEOMS = [(2, 1, 1), (3, 2, 1), (33, 3, 3), (65, 5, 9), (97, 7, 17)]


def _data(C, P, S, seed):
    th = theta_uniform(P)
    rng = np.random.default_rng(seed)
    return th, O.angle_table(th), rng.uniform(0.5, 2.0, (P, S, C)).astype(np.float32)


def _params(alg):
    return {"beta": 0.3} if alg in ("pml", "apmlr") else {}


def _close(got, want, tol):
    """Pixels no ray crosses (total length 0, possible with one or two
    angles) are 0/0 = NaN in the reference's update: NaN in the same places,
    relative L2 over the rest."""
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(got), nan)
    if (~nan).any():
        assert rel_l2(got[~nan], want[~nan]) < tol


@pytest.mark.parametrize("C,P,S", GEOMS)
@pytest.mark.parametrize("alg", ["sirt", "mlem", "pml", "apmlr"])
def test_small_and_ragged_geometries_exact(C, P, S, alg):
    th, tabs, sino = _data(C, P, S, C * 7 + P)
    kw = _params(alg)
    ref = O.run(alg, sino, tables=tabs, n_iter=2, **kw)["recon"]
    for K in (1, 4):
        plan = tg.Plan(P, S, C, th, slices_per_pass=K)
        plan.set_sinogram(sino, apply_abs=alg != "sirt")
        plan.reset_recon(alg)
        plan.iterate(alg, 2, tg.default_params(alg, **kw))
        _close(plan.get_recon(alg), ref, 2e-6)
        plan.close()


@pytest.mark.parametrize("C,P,S", GEOMS)
@pytest.mark.parametrize("alg", ["sirt", "pml"])
def test_small_and_ragged_geometries_fast_tiles(C, P, S, alg):
    """The measured fast path (16-bit lengths, 8 slices per pass, tile-staged
    forward, half gathers, two streams when there are two batches) on
    geometries smaller than one tile, one ray group or one batch. With so
    few angles a half factor's rounding (2^-11) is not averaged over many
    rays per pixel, hence the 1e-3 bound here against 1e-4 at 72+ angles."""
    th, tabs, sino = _data(C, P, S, C * 11 + P)
    kw = _params(alg)
    ref = O.run(alg, sino, tables=tabs, n_iter=2, precision=O.F64, **kw)["recon"]
    for side in (32, 96):
        plan = tg.Plan(P, S, C, th, slices_per_pass=8, mode="fast", len_storage="u16",
                       delta_index=True, forward_tiles=True, half_gathers=True,
                       forward_tile_side=side, backward_tile_width=16)
        plan.set_sinogram(sino, apply_abs=alg != "sirt")
        plan.reset_recon(alg)
        plan.iterate(alg, 2, tg.default_params(alg, **kw))
        _close(plan.get_recon(alg), ref, 1e-3)
        plan.close()
