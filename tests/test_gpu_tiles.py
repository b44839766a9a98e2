"""Tile-staged forward projection (fast mode, forward_tiles=1) against the
ray-ordered fast path and the FP64 oracle."""
import numpy as np
import pytest

import trace_gb300 as tg
from oracle import oracle as O
from tests._util import bits, rel_l2, theta_uniform

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


@pytest.mark.parametrize("alg", ["sirt", "mlem", "pml", "apmlr"])
@pytest.mark.parametrize("K,S", [(4, 4), (8, 9)])
def test_half_gathers_against_fp64(alg, K, S):
    """16-bit gather operands (shared-memory tile and ratio factors as halves,
    FP32 arithmetic): error against the FP64 oracle stays at the level of the
    16-bit lengths. Small grids converge from far away in few iterations, the
    loosest case for half factors (rel-L2 bound 1e-4 here; the 2048^2 x 1500
    workload's 30-iteration error is measured by the benchmark). The first
    iteration stores halves of the factors, later ones of factor - 1."""
    C, P, it = 96, 72, 6
    th = theta_uniform(P)
    tabs = O.angle_table(th)
    from trace_gb300.phantom import ellipse_phantoms
    sino = O.forward(ellipse_phantoms(C, S, seed=5, texture_sigma=0.02), tabs)
    kw = dict(beta=0.05) if alg in ("pml", "apmlr") else {}
    ref = O.run(alg, sino, tables=tabs, n_iter=it, precision=O.F64, **kw)["recon"]
    prm = tg.default_params(alg, beta=0.05)
    errs = {}
    for half in (False, True):
        plan = tg.Plan(P, S, C, th, slices_per_pass=K, mode="fast", len_storage="u16",
                       delta_index=True, forward_tiles=True, half_gathers=half)
        plan.set_sinogram(sino, apply_abs=alg != "sirt")
        plan.reset_recon(alg)
        plan.iterate(alg, it, prm)
        errs[half] = rel_l2(plan.get_recon(alg), ref)
        plan.close()
    assert errs[False] < 1e-4, errs
    assert errs[True] < 1e-4, errs


@pytest.mark.parametrize("alg", ["mlem", "pml"])
def test_first_iteration_half_factors(alg):
    """The first iteration after a reset stores halves of the factors
    themselves (factors lie anywhere in (0, max) there), later iterations
    halves of factor - 1: each of the first two iterations stays within
    1e-4 relative L2 of the FP64 oracle, and a reset starts the sequence
    again with the same bits."""
    C, P, S = 96, 72, 8
    th = theta_uniform(P)
    tabs = O.angle_table(th)
    from trace_gb300.phantom import ellipse_phantoms
    sino = O.forward(ellipse_phantoms(C, S, seed=9, texture_sigma=0.02), tabs)
    kw = dict(beta=0.05) if alg == "pml" else {}
    prm = tg.default_params(alg, beta=0.05)
    plan = tg.Plan(P, S, C, th, slices_per_pass=8, mode="fast", len_storage="u16",
                   delta_index=True, forward_tiles=True, half_gathers=True)
    plan.set_sinogram(sino, apply_abs=True)
    plan.reset_recon(alg)
    got = []
    for it in (1, 2):
        ref = O.run(alg, sino, tables=tabs, n_iter=it, precision=O.F64, **kw)["recon"]
        plan.iterate(alg, 1, prm)
        got.append(plan.get_recon(alg))
        assert rel_l2(got[-1], ref) < 1e-4, (alg, it)
    plan.reset_recon(alg)
    plan.iterate(alg, 1, prm)
    assert np.array_equal(bits(plan.get_recon(alg)), bits(got[0]))
    plan.close()


def test_half_gathers_keep_operator_path_fp32():
    """tg_reduce (the reference's RunParallelReduction) runs the tile-ordered
    forward with FP32 factors on a half_gathers plan (half tile, f16 lengths
    in the backward matrix), so its replica agrees with the plain tiled
    plan's to the rounding of those operands (relative L2 <= 1e-4)."""
    C, P, S = 64, 40, 4
    th = theta_uniform(P)
    rng = np.random.default_rng(7)
    sino = rng.uniform(0.5, 2.0, (P, S, C)).astype(np.float32)
    prm = tg.default_params("pml", beta=0.1)
    reps = []
    for half in (False, True):
        plan = tg.Plan(P, S, C, th, slices_per_pass=4, mode="fast", len_storage="u16",
                       delta_index=True, forward_tiles=True, half_gathers=half)
        plan.set_sinogram(sino, apply_abs=True)
        plan.reset_recon("pml")
        plan.reduce("pml", prm)
        reps.append(plan.get_replica("pml"))
        plan.close()
    assert rel_l2(reps[1], reps[0]) < 1e-4


@pytest.mark.parametrize("kw", [dict(mode="fast"), dict(mode="exact", forward_tiles=True),
                                dict(mode="fast", forward_tiles=True, backward_staged=True)])
def test_half_gathers_needs_tiles_and_l1_backprojection(kw):
    with pytest.raises(tg.TraceError) as e:
        tg.Plan(8, 1, 16, theta_uniform(8), half_gathers=True, **kw)
    assert e.value.status == 1


@pytest.mark.parametrize("alg", ["mlem", "pml", "apmlr"])
def test_sixteen_slices_per_pass_match_eight(alg):
    C, P, S = 96, 72, 19
    th = theta_uniform(P)
    tabs = O.angle_table(th)
    from trace_gb300.phantom import ellipse_phantoms
    sino = O.forward(ellipse_phantoms(C, S, seed=17, texture_sigma=0.02), tabs)
    prm = tg.default_params(alg, beta=0.05)
    outs = []
    for K in (8, 16):
        plan = tg.Plan(P, S, C, th, slices_per_pass=K, mode="fast", len_storage="u16",
                       delta_index=True, forward_tiles=True, half_gathers=True)
        plan.set_sinogram(sino, apply_abs=True)
        plan.reset_recon(alg)
        plan.iterate(alg, 4, prm)
        outs.append(plan.get_recon(alg))
        plan.close()
    # same arithmetic and summation order per slice
    assert np.array_equal(bits(outs[1]), bits(outs[0]))


def test_sixteen_slices_with_tiles_need_half_gathers():
    with pytest.raises(tg.TraceError) as e:
        tg.Plan(8, 16, 16, theta_uniform(8), slices_per_pass=16, mode="fast",
                forward_tiles=True)
    assert e.value.status == 1


@pytest.mark.parametrize("storage", ["f32", "f16", "bf16", "u16"])
def test_half_gathers_with_each_length_storage(storage):
    """Half gathers over every forward length storage: 16-bit storages keep
    f16 lengths in the backward matrix (the FMA operands as stored), f32
    storage keeps f32 lengths there and rounds them per FMA."""
    C, P, S, it = 80, 60, 8, 5
    th = theta_uniform(P)
    tabs = O.angle_table(th)
    from trace_gb300.phantom import ellipse_phantoms
    sino = O.forward(ellipse_phantoms(C, S, seed=9, texture_sigma=0.02), tabs)
    ref = O.run("mlem", sino, tables=tabs, n_iter=it, precision=O.F64)["recon"]
    plan = tg.Plan(P, S, C, th, slices_per_pass=8, mode="fast", len_storage=storage,
                   delta_index=True, forward_tiles=True, half_gathers=True)
    plan.set_sinogram(sino, apply_abs=True)
    plan.reset_recon("mlem")
    plan.iterate("mlem", it, tg.default_params("mlem"))
    err = rel_l2(plan.get_recon("mlem"), ref)
    plan.close()
    assert err < (3e-3 if storage == "bf16" else 1e-4), err


@pytest.mark.parametrize("alg", ["sirt", "mlem", "pml", "apmlr"])
def test_operator_path_uses_tiles(alg):
    """reduce -> replica and forward_project on a tile-ordered plan agree with
    the ray-ordered plan of the same storage (ray sums regrouped by tile
    runs: relative L2 <= 1e-6), as the drivers' RunParallelReduction /
    UpdateRecon loop
    calls them."""
    C, P, S = 72, 54, 6
    th = theta_uniform(P)
    rng = np.random.default_rng(17)
    sino = rng.uniform(0.5, 2.0, (P, S, C)).astype(np.float32)
    prm = tg.default_params(alg, beta=0.1)
    reps, sims, recons = [], [], []
    for tiles in (False, True):
        plan = tg.Plan(P, S, C, th, slices_per_pass=2, mode="fast", len_storage="u16",
                       delta_index=True, forward_tiles=tiles)
        plan.set_sinogram(sino, apply_abs=alg != "sirt")
        plan.reset_recon(alg)
        for _ in range(2):  # reference driver loop: Reduce, then UpdateRecon
            plan.reduce(alg, prm)
            if alg in ("pml", "apmlr"):
                plan.calculate_fg(alg, prm)
            plan.update_recon(alg, prm)
        reps.append(plan.get_replica(alg))
        recons.append(plan.get_recon(alg))
        sims.append(plan.forward_project(alg))
        plan.close()
    assert rel_l2(reps[1], reps[0]) < 1e-6
    assert rel_l2(recons[1], recons[0]) < 1e-6
    assert rel_l2(sims[1], sims[0]) < 1e-6


@pytest.mark.parametrize("alg", ["sirt", "mlem", "pml"])
@pytest.mark.parametrize("storage,half", [("f32", False), ("u16", True)])
def test_compensated_sums_against_fp64(alg, storage, half):
    """compensated=1 (Kahan ray sums over 8-segment blocks and across tile
    runs, Kahan pixel sums over 4-angle blocks): within 1e-4 of the FP64
    oracle like the plain sums and bit-reproducible; with f32 storage, where
    summation is the error left, no further from FP64 than the plain sums
    (beyond 1e-7 of slack); with 16-bit storage, whose quantisation
    dominates, within 5 % of their error."""
    C, P, S, it = 128, 120, 8, 6
    th = theta_uniform(P)
    tabs = O.angle_table(th)
    from trace_gb300.phantom import ellipse_phantoms
    sino = O.forward(ellipse_phantoms(C, S, seed=21, texture_sigma=0.02), tabs)
    kw = dict(beta=0.05) if alg == "pml" else {}
    ref = O.run(alg, sino, tables=tabs, n_iter=it, precision=O.F64, **kw)["recon"]
    prm = tg.default_params(alg, beta=0.05)
    outs = {}
    for comp in (False, True, True):
        plan = tg.Plan(P, S, C, th, slices_per_pass=8, mode="fast", len_storage=storage,
                       delta_index=True, forward_tiles=True, half_gathers=half,
                       compensated=comp)
        plan.set_sinogram(sino, apply_abs=alg != "sirt")
        plan.reset_recon(alg)
        plan.iterate(alg, it, prm)
        out = plan.get_recon(alg)
        plan.close()
        if comp in outs:
            assert np.array_equal(bits(out), bits(outs[comp]))
        outs[comp] = out
    e_plain, e_comp = rel_l2(outs[False], ref), rel_l2(outs[True], ref)
    assert e_comp < 1e-4, (e_plain, e_comp)
    if storage == "f32":
        assert e_comp <= e_plain + 1e-7, (e_plain, e_comp)
    else:
        assert abs(e_comp - e_plain) <= 0.05 * e_plain, (e_plain, e_comp)


@pytest.mark.parametrize("kw", [dict(mode="exact", forward_tiles=False),
                                dict(mode="fast", forward_tiles=False),
                                dict(mode="fast", forward_tiles=True, backward_staged=True)])
def test_compensated_needs_tiles_and_l1_backprojection(kw):
    with pytest.raises(tg.TraceError) as e:
        tg.Plan(8, 1, 16, theta_uniform(8), compensated=True, **kw)
    assert e.value.status == 1


@pytest.mark.parametrize("kw", [dict(mode="exact"),
                                dict(mode="fast", len_storage="u16", delta_index=True,
                                     slices_per_pass=8, forward_tiles=True,
                                     half_gathers=True)])
@pytest.mark.parametrize("alg", ["sirt", "mlem", "pml", "apmlr"])
def test_backward_tile_shapes_are_bit_identical(kw, alg):
    """The backprojection's pixel tile (8x4 default, 16x2, 4x8) only decides
    which warp owns a pixel; every pixel sums its angles in the same order,
    so the results are bit-identical (an odd grid, uneven tiles)."""
    C, P, S = 99, 70, 5
    th = theta_uniform(P)
    rng = np.random.default_rng(41)
    sino = rng.uniform(0.5, 2.0, (P, S, C)).astype(np.float32)
    prm = tg.default_params(alg, beta=0.2)
    outs = []
    for tw in (0, 16, 4):
        plan = tg.Plan(P, S, C, th, backward_tile_width=tw, **kw)
        plan.set_sinogram(sino, apply_abs=alg != "sirt")
        plan.reset_recon(alg)
        plan.iterate(alg, 3, prm)
        outs.append(plan.get_recon(alg))
        plan.close()
    assert np.array_equal(bits(outs[1]), bits(outs[0]))
    assert np.array_equal(bits(outs[2]), bits(outs[0]))


@pytest.mark.parametrize("ts", [32, 48, 80, 96])
@pytest.mark.parametrize("alg", ["sirt", "mlem", "pml"])
def test_forward_tile_sides(ts, alg):
    """Forward tiles of 32 to 96 pixels regroup each ray's sum by tile runs:
    within 1e-6 of the 64-pixel tiles with FP32 operands, and the benchmark
    configuration stays within 1e-4 of the FP64 oracle."""
    C, P, S, it = 200, 150, 8, 5
    th = theta_uniform(P)
    tabs = O.angle_table(th)
    from trace_gb300.phantom import ellipse_phantoms
    sino = O.forward(ellipse_phantoms(C, S, seed=23, texture_sigma=0.02), tabs)
    kw = dict(beta=0.05) if alg == "pml" else {}
    ref = O.run(alg, sino, tables=tabs, n_iter=it, precision=O.F64, **kw)["recon"]
    prm = tg.default_params(alg, beta=0.05)
    res = {}
    for side in (0, ts):
        for half in (False, True):
            if side == 96 and not half:
                continue  # an f32 tile of 96 x 97 x 8 would not fit shared memory
            plan = tg.Plan(P, S, C, th, slices_per_pass=8, mode="fast", len_storage="u16",
                           delta_index=True, forward_tiles=True, half_gathers=half,
                           forward_tile_side=side)
            plan.set_sinogram(sino, apply_abs=alg != "sirt")
            plan.reset_recon(alg)
            plan.iterate(alg, it, prm)
            res[(side, half)] = plan.get_recon(alg)
            plan.close()
    if (ts, False) in res:
        assert rel_l2(res[(ts, False)], res[(0, False)]) < 1e-6
    assert rel_l2(res[(ts, True)], ref) < 1e-4


def test_forward_tile_that_does_not_fit_is_rejected():
    with pytest.raises(tg.TraceError) as e:
        tg.Plan(8, 8, 100, theta_uniform(8), slices_per_pass=8, mode="fast",
                forward_tiles=True, forward_tile_side=96)  # f32 tile: 298 KB
    assert e.value.status == 1
    for side in (40, 112):  # not a multiple of 16; beyond the one-byte step
        with pytest.raises(tg.TraceError) as e:
            tg.Plan(8, 1, 100, theta_uniform(8), mode="fast", forward_tiles=True,
                    forward_tile_side=side)
        assert e.value.status == 1


@pytest.mark.parametrize("warps", [8, 16])
def test_forward_block_warps_are_bit_identical(warps):
    """Fewer warps per forward tile block (runs in flight per tile) change
    only the schedule: every run is still one lane's FMA chain into its own
    slot, so the results are the same bits."""
    C, P, S = 150, 100, 8
    th = theta_uniform(P)
    rng = np.random.default_rng(43)
    sino = rng.uniform(0.5, 2.0, (P, S, C)).astype(np.float32)
    prm = tg.default_params("pml", beta=0.1)
    outs = []
    for w in (0, warps):
        plan = tg.Plan(P, S, C, th, slices_per_pass=8, mode="fast", len_storage="u16",
                       delta_index=True, forward_tiles=True, half_gathers=True,
                       forward_block_warps=w)
        plan.set_sinogram(sino, apply_abs=True)
        plan.reset_recon("pml")
        plan.iterate("pml", 3, prm)
        outs.append(plan.get_recon("pml"))
        plan.close()
    assert np.array_equal(bits(outs[1]), bits(outs[0]))


@pytest.mark.parametrize("case", ["center", "apmlr_inner", "apmlr_top", "apmlr_bottom"])
def test_fast_tiles_geometry_variants_against_fp64(case):
    """The measured fast path (16-bit lengths, 8 slices per pass, tile-staged
    forward, half gathers) with a rotation centre off the middle, and APMLR
    on slabs of a larger volume (inner, top and bottom: the axial penalty's
    boundary cases), against the FP64 oracle run on the same slab."""
    C, P, S = 96, 72, 9
    th = theta_uniform(P)
    tabs = O.angle_table(th)
    from trace_gb300.phantom import ellipse_phantoms
    center = C / 2 + 3.5 if case == "center" else 0.0
    alg = "pml" if case == "center" else "apmlr"
    slab = {"center": (0, S), "apmlr_inner": (9, 40), "apmlr_top": (0, 40),
            "apmlr_bottom": (31, 40)}[case]
    sino = O.forward(ellipse_phantoms(C, S, seed=23, texture_sigma=0.02), tabs,
                     center=center)
    kw = dict(beta=0.05) if alg == "pml" else dict(beta=0.05, beta1=0.5)
    ref = O.run(alg, sino, tables=tabs, n_iter=4, precision=O.F64, center=center,
                slice_id=slab[0], num_total_slices=slab[1], **kw)["recon"]
    plan = tg.Plan(P, S, C, th, center=center, slice_id=slab[0], num_total_slices=slab[1],
                   slices_per_pass=8, mode="fast", len_storage="u16", delta_index=True,
                   forward_tiles=True, half_gathers=True)
    plan.set_sinogram(sino, apply_abs=True)
    plan.reset_recon(alg)
    plan.iterate(alg, 4, tg.default_params(alg, **kw))
    assert rel_l2(plan.get_recon(alg), ref) < 1e-4, case
    plan.close()
