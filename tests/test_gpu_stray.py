"""Geometries where the reference's tracer emits a stray segment: at the
angle nearest to 90 degrees, an edge ray gets one 1/16-long segment on the
far side of the grid (float rounding with the source a million units away).
868 columns x 1129 angles is the smallest such geometry found (angle 564,
column 1). The segment is outside its pixel's two-column backward window
(kept in the plan's exception list) and its step breaks the 4-bit code (the
ray-ordered delta form falls back to tracing on the fly); results must still
match the reference's algorithm."""
import numpy as np
import pytest

import trace_gb300 as tg
from oracle import oracle as O
from tests._util import bits, rel_l2, theta_uniform

pytestmark = pytest.mark.gpu

C, P = 868, 1129


@pytest.fixture(scope="module")
def data():
    th = theta_uniform(P)
    tabs = O.angle_table(th)
    from trace_gb300.phantom import ellipse_phantoms
    ph = ellipse_phantoms(C, 1, seed=41)
    sino = O.forward(ph, tabs, threads=16)
    return th, tabs, ph, sino


def test_stray_segment_is_traced_like_the_reference(data):
    th, tabs, _, _ = data
    counts, offs, idx, ln, _ = O.trace(C, tuple(t[564:565] for t in tabs), threads=8)
    ray = offs[1], offs[2]  # column 1
    far = idx[ray[0]:ray[1]] % C
    assert far.min() == 0 and far.max() >= C - 2  # one segment on the far side
    plan = tg.Plan(P, 1, C, th, slices_per_pass=1, mode="fast", len_storage="u16",
                   delta_index=True, forward_tiles=True, half_gathers=True)
    info = plan.info()
    assert info["window_exceptions"] >= 1 and info["forward_traced"] == 1
    plan.close()


def test_exact_mode_with_stray_segments(data):
    th, tabs, ph, sino = data
    plan = tg.Plan(P, 1, C, th)
    assert plan.info()["window_exceptions"] >= 1
    plan.set_recon("sirt", ph)
    sim = plan.forward_project("sirt")
    assert np.array_equal(bits(sim), bits(sino))
    # SIRT and MLEM: the reference's float PML root cancels at this size, so
    # reassociated sums drift apart there (PML is checked against FP64 below)
    for alg in ("sirt", "mlem"):
        ref = O.run(alg, sino, tables=tabs, n_iter=2, threads=16)["recon"]
        plan.set_sinogram(sino, apply_abs=alg != "sirt")
        plan.reset_recon(alg)
        plan.iterate(alg, 2)
        assert rel_l2(plan.get_recon(alg), ref) < 2e-6, alg
    plan.close()


@pytest.mark.parametrize("alg", ["mlem", "pml"])
def test_fast_paths_with_stray_segments_against_fp64(data, alg):
    th, tabs, _, sino = data
    kw_alg = dict(beta=0.1) if alg == "pml" else {}
    ref = O.run(alg, sino, tables=tabs, n_iter=3, precision=O.F64, threads=16,
                **kw_alg)["recon"]
    for kw in (dict(len_storage="u16", delta_index=True, forward_tiles=True, half_gathers=True),
               dict(len_storage="u16", delta_index=True),
               dict(len_storage="f32", backward_staged=True)):
        plan = tg.Plan(P, 1, C, th, mode="fast", **kw)
        plan.set_sinogram(sino, apply_abs=True)
        plan.reset_recon(alg)
        plan.iterate(alg, 3, tg.default_params(alg, beta=0.1))
        assert rel_l2(plan.get_recon(alg), ref) < 1e-4, kw
        plan.close()


def test_out_of_grid_stray_segment_is_dropped():
    """At 2048 columns x 1065 angles the reference's tracer gives the last
    angle's edge ray a 1/16-long segment whose cell index is one row past
    the grid (the reference would index out of bounds). Both the device
    tracer and the oracle drop it; everything else matches."""
    C2, P2 = 2048, 1065
    th = theta_uniform(P2)
    tabs = O.angle_table(th)
    counts, offs, idx, ln, _, _ = O.ref_trace(C2, th[[P2 - 1]]) if O.ref() else (None,) * 6
    if idx is not None:
        assert ((idx < 0) | (idx >= C2 * C2)).sum() == 1
    from trace_gb300.phantom import ellipse_phantoms
    ph = ellipse_phantoms(C2, 1, seed=43)
    sino = O.forward(ph, tabs, threads=16)
    plan = tg.Plan(P2, 1, C2, th)
    cnt = plan.trace_rays(counts_only=True)
    ocnt, *_ = O.trace(C2, tuple(t[P2 - 1:] for t in tabs), threads=8)
    assert np.array_equal(cnt[(P2 - 1) * C2:], ocnt)
    plan.set_recon("sirt", ph)
    assert np.array_equal(bits(plan.forward_project("sirt")), bits(sino))
    plan.close()


def test_fp64_mode_with_stray_segments(data):
    th, tabs, _, sino = data
    ref = O.run("sirt", sino, tables=tabs, n_iter=2, precision=O.F64, threads=16)["recon"]
    plan = tg.Plan(P, 1, C, th, mode="fp64")
    plan.set_sinogram(sino)
    plan.reset_recon("sirt")
    plan.iterate("sirt", 2)
    assert rel_l2(plan.get_recon("sirt"), ref) < 1e-6
    plan.close()
