"""Parity of the benchmarked configurations at benchmark-like sizes.

  * the mixed-precision batched path exactly as the benchmark runs it (16-bit
    fixed-point lengths, f16 gather operands, 8 slices per matrix pass,
    tile-staged forward, fast arithmetic) against the CPU FP64 oracle of the
    same algorithm: relative L2 <= 1e-4 after every one of 30 iterations,
    PML (beta 0.05, textured phantoms) and MLEM (Poisson data, sinogram
    floor 1e-6), at 512 x 512 x 360 angles, 8 slices;
  * exact mode at the SIRT 256 workload (256 x 256, 180 angles, 8 slices,
    10 iterations, Poisson I0 = 1e4) against the oracle, which is pinned bit
    for bit to the compiled reference at this workload: relative L2 <= 2e-6
    per iteration;
  * the tile-staged forward is deterministic: identical plans give
    identical bits.
"""
import os

import numpy as np
import pytest

import trace_gb300 as tg
from oracle import oracle as O
from tests._util import CONFIG1, bits, config1_data, rel_l2, theta_uniform

pytestmark = pytest.mark.gpu

BENCH_PLAN = dict(len_storage="u16", slices_per_pass=8, mode="fast", delta_index=True,
                  forward_tiles=True, half_gathers=True)


def _mid_data(alg):
    from trace_gb300.phantom import ellipse_phantoms, poisson_log
    C, P, S = 512, 360, 8
    th = theta_uniform(P)
    tabs = O.angle_table(th)
    threads = os.cpu_count() or 8
    if alg == "pml":
        ph = ellipse_phantoms(C, S, seed=31, texture_sigma=0.02)
        sino = O.forward(ph, tabs, threads=threads)
        clip = None
    else:
        ph = ellipse_phantoms(C, S, seed=32)
        sino = poisson_log(O.forward(ph, tabs, threads=threads), 5e3, seed=33, g=C)
        clip = 1e-6
        sino = np.maximum(np.abs(sino), np.float32(clip))
    return th, tabs, np.ascontiguousarray(sino, np.float32), clip, threads


@pytest.mark.parametrize("alg", ["pml", "mlem"])
def test_benchmark_configuration_within_1e4_of_fp64(alg):
    th, tabs, sino, clip, threads = _mid_data(alg)
    P, S, C = sino.shape
    n_iter = 30
    kw = dict(beta=0.05) if alg == "pml" else {}
    ref = O.run(alg, sino, tables=tabs, n_iter=n_iter, precision=O.F64, threads=threads,
                want_iters=True, **kw)["iters"]
    plan = tg.Plan(P, S, C, th, **BENCH_PLAN)
    plan.set_sinogram(sino, apply_abs=True, clip_min=clip)
    plan.reset_recon(alg)
    prm = tg.default_params(alg, beta=0.05)
    errs = []
    for it in range(n_iter):
        plan.iterate(alg, 1, prm)
        errs.append(rel_l2(plan.get_recon(alg), ref[it]))
    plan.close()
    assert max(errs) <= 1e-4, errs


@pytest.mark.parametrize("K", [1, 8])
def test_exact_mode_at_sirt256_workload(K):
    th, tabs, sino = config1_data()
    c = CONFIG1
    want = O.run("sirt", sino, tables=tabs, n_iter=c["n_iter"], threads=1,
                 want_iters=True)["iters"]
    plan = tg.Plan(c["P"], c["S"], c["C"], th, sin_tab=tabs[0], cos_tab=tabs[1],
                   slices_per_pass=K)
    plan.set_sinogram(sino)
    plan.reset_recon("sirt")
    for it in range(c["n_iter"]):
        plan.iterate("sirt", 1)
        err = rel_l2(plan.get_recon("sirt"), want[it])
        assert err <= 2e-6, (it, err)
    plan.close()


@pytest.mark.parametrize("alg", ["sirt", "mlem", "pml"])
def test_tiled_forward_is_deterministic(alg):
    C, P, S = 192, 150, 9
    th = theta_uniform(P)
    rng = np.random.default_rng(5)
    sino = rng.uniform(0.5, 2.0, (P, S, C)).astype(np.float32)
    prm = tg.default_params(alg, beta=0.05)
    outs, sims = [], []
    for _ in range(2):
        plan = tg.Plan(P, S, C, th, **BENCH_PLAN)
        plan.set_sinogram(sino, apply_abs=alg != "sirt")
        plan.reset_recon(alg)
        plan.iterate(alg, 4, prm)
        outs.append(plan.get_recon(alg))
        sims.append(plan.forward_project(alg))
        plan.close()
    assert np.array_equal(bits(outs[0]), bits(outs[1]))
    assert np.array_equal(bits(sims[0]), bits(sims[1]))
