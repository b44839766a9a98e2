"""Forward projection with rays traced on the fly (forward_on_the_fly=1, no
stored ray-ordered forward matrix) against the stored-matrix path: the same
float lengths summed in the same order, so results are bit-identical to the
f32 stored form in both arithmetic modes."""
import numpy as np
import pytest

import trace_gb300 as tg
from tests._util import bits, ellipse_sino, rel_l2, theta_uniform
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode,K", [("exact", 1), ("exact", 4), ("fast", 8), ("fast", 2)])
def test_on_the_fly_forward_projection_bit_identical(mode, K):
    C, P, S = 100, 70, 5
    th, tabs, ph, _ = ellipse_sino(C, P, S, seed=21)
    outs = []
    for otf in (False, True):
        plan = tg.Plan(P, S, C, th, slices_per_pass=K, mode=mode, forward_on_the_fly=otf)
        plan.set_recon("sirt", ph)
        outs.append(plan.forward_project("sirt"))
        info = plan.info()
        assert (info["forward_bytes"] == 0) == otf
        plan.close()
    assert np.array_equal(bits(outs[0]), bits(outs[1]))


@pytest.mark.parametrize("alg", ["sirt", "mlem", "pml", "apmlr"])
@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_on_the_fly_iterations_bit_identical(alg, mode):
    C, P, S = 96, 60, 4
    th, tabs, _, sino = ellipse_sino(C, P, S, seed=5)
    prm = tg.default_params(alg, beta=0.1)
    outs = []
    for otf in (False, True):
        plan = tg.Plan(P, S, C, th, slices_per_pass=2, mode=mode, forward_on_the_fly=otf)
        plan.set_sinogram(sino, apply_abs=alg != "sirt")
        plan.reset_recon(alg)
        plan.iterate(alg, 3, prm)
        outs.append(plan.get_recon(alg))
        plan.close()
    assert np.array_equal(bits(outs[0]), bits(outs[1]))
    if mode == "exact":
        kw = dict(beta=0.1) if alg in ("pml", "apmlr") else {}
        ref = O.run(alg, sino, tables=tabs, n_iter=3, **kw)["recon"]
        assert rel_l2(outs[1], ref) < 2e-6


def test_on_the_fly_operator_path_and_memory():
    C, P, S = 128, 90, 3
    th, tabs, _, sino = ellipse_sino(C, P, S, seed=9)
    prm = tg.default_params("pml", beta=0.1)
    reps, dev = [], []
    for otf in (False, True):
        plan = tg.Plan(P, S, C, th, forward_on_the_fly=otf)
        plan.set_sinogram(sino, apply_abs=True)
        plan.reset_recon("pml")
        plan.reduce("pml", prm)
        reps.append(plan.get_replica("pml"))
        dev.append(plan.info()["device_bytes"])
        plan.close()
    assert np.array_equal(bits(reps[0]), bits(reps[1]))
    assert dev[1] < dev[0]


def test_on_the_fly_with_tiles_and_half_gathers():
    """The tile stream is built from the stored delta-coded matrix, the stored
    explicit-index matrix, or by tracing (no stored matrix): all three give
    the same reconstruction."""
    C, P, S = 96, 72, 8
    th, tabs, _, sino = ellipse_sino(C, P, S, seed=13)
    prm = tg.default_params("pml", beta=0.05)
    outs = []
    for delta, otf in ((True, False), (True, True), (False, False)):
        plan = tg.Plan(P, S, C, th, slices_per_pass=8, mode="fast", len_storage="u16",
                       delta_index=delta, forward_tiles=True, half_gathers=True,
                       forward_on_the_fly=otf)
        plan.set_sinogram(sino, apply_abs=True)
        plan.reset_recon("pml")
        plan.iterate("pml", 4, prm)
        outs.append(plan.get_recon("pml"))
        plan.close()
    # the tiled forward's run sums are added atomically: order may differ
    assert rel_l2(outs[1], outs[0]) < 1e-6
    assert rel_l2(outs[2], outs[0]) < 1e-6


def test_on_the_fly_rejected_in_fp64_mode():
    with pytest.raises(tg.TraceError) as e:
        tg.Plan(8, 1, 16, theta_uniform(8), mode="fp64", forward_on_the_fly=True)
    assert e.value.status == 1
