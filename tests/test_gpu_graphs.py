"""CUDA-graph replay of iterations and batches of independent plans: the
results must be bit-identical to plain launches, in exact mode and on the
tile-staged fast path (no atomics: every launch sums in the same order)."""
import numpy as np
import pytest

import trace_gb300 as tg
from tests._util import bits, theta_uniform

pytestmark = pytest.mark.gpu


def _plan(C, P, S, seed, alg, **kw):
    rng = np.random.default_rng(seed)
    sino = rng.uniform(0.5, 2.0, (P, S, C)).astype(np.float32)
    plan = tg.Plan(P, S, C, theta_uniform(P), **kw)
    plan.set_sinogram(sino, apply_abs=alg != "sirt")
    plan.reset_recon(alg)
    return plan


@pytest.mark.parametrize("alg", ["sirt", "pml", "apmlr"])
@pytest.mark.parametrize("kw", [dict(slices_per_pass=2),
                                dict(slices_per_pass=4, mode="fast", len_storage="u16",
                                     delta_index=True, forward_tiles=True)])
def test_graph_replay_identical(alg, kw):
    prm = tg.default_params(alg, beta=0.3)
    outs = []
    for graphs in (False, True):
        plan = _plan(64, 48, 5, 1, alg, **kw)
        plan.set_graphs(graphs)
        plan.iterate(alg, 3, prm)
        plan.iterate(alg, 2, prm)  # parity flips between calls
        outs.append(plan.get_recon(alg))
        plan.close()
    # the tile-staged forward adds each ray's run sums in a fixed order
    assert np.array_equal(bits(outs[0]), bits(outs[1]))


def test_batch_matches_individual_plans():
    specs = [(64, 40, 3, "sirt"), (96, 70, 2, "mlem"), (48, 33, 5, "pml"),
             (80, 25, 1, "mlem"), (64, 90, 4, "sirt")]
    prms = [tg.default_params(a, beta=0.4) for *_, a in specs]
    singles = []
    for i, (C, P, S, alg) in enumerate(specs):
        plan = _plan(C, P, S, 10 + i, alg, slices_per_pass=2)
        plan.iterate(alg, 4, prms[i])
        singles.append(plan.get_recon(alg))
        plan.close()
    plans = [_plan(C, P, S, 10 + i, alg, slices_per_pass=2)
             for i, (C, P, S, alg) in enumerate(specs)]
    batch = tg.Batch(plans)
    batch.iterate([a for *_, a in specs], 3, prms)
    batch.iterate([a for *_, a in specs], 1, prms)
    for plan, (C, P, S, alg), want in zip(plans, specs, singles):
        assert np.array_equal(bits(plan.get_recon(alg)), bits(want))
    batch.close()
    for p in plans:
        p.close()


def test_plans_created_from_host_threads():
    """Plans created and iterated concurrently from several host threads
    (each plan traces on its own stream) give the same results as plans
    created one after another (exact mode: bit-identical)."""
    from concurrent.futures import ThreadPoolExecutor
    cases = [(64, 48, 3, 11, "sirt"), (96, 40, 2, 12, "mlem"), (80, 60, 4, 13, "pml"),
             (48, 36, 5, 14, "apmlr"), (72, 30, 1, 15, "sirt"), (56, 64, 3, 16, "mlem")]

    def run(case):
        C, P, S, seed, alg = case
        plan = _plan(C, P, S, seed, alg, slices_per_pass=1)
        plan.iterate(alg, 2, tg.default_params(alg, beta=0.3))
        out = plan.get_recon(alg)
        plan.close()
        return out

    serial = [run(c) for c in cases]
    with ThreadPoolExecutor(4) as ex:
        threaded = list(ex.map(run, cases))
    for a, b in zip(serial, threaded):
        assert np.array_equal(bits(a), bits(b))


MULTI_SPECS = [  # (C, P, S, alg, slices per pass, half gathers, compensated)
    (64, 40, 3, "sirt", 2, True, False), (96, 70, 9, "mlem", 8, True, False),
    (48, 33, 5, "pml", 4, True, False), (80, 25, 1, "mlem", 1, False, False),
    (130, 90, 16, "sirt", 16, True, False), (72, 61, 7, "apmlr", 4, True, False),
    (100, 45, 6, "mlem", 8, True, True), (64, 50, 4, "pml", 4, False, True),
]


def test_batch_multi_plan_launches_match_individual_plans():
    """Fast tile-staged plans with 16-bit lengths advance together through the
    multi-plan launches (one per kernel variant and slice-batch round, blocks
    walking every plan's work): bit-identical to each plan iterated alone,
    from a fresh reconstruction (first iteration: halves of the factors) on, across
    calls (buffer parity), with far fewer launches than per-plan kernels."""
    def mk(i, spec):
        C, P, S, alg, K, half, comp = spec
        return _plan(C, P, S, 30 + i, alg, slices_per_pass=K, mode="fast",
                     len_storage="u16", delta_index=True, forward_tiles=True,
                     half_gathers=half, compensated=comp)
    algs = [s[3] for s in MULTI_SPECS]
    prms = [tg.default_params(a, beta=0.4) for a in algs]
    singles = []
    for i, spec in enumerate(MULTI_SPECS):
        plan = mk(i, spec)
        plan.iterate(algs[i], 4, prms[i])
        singles.append(plan.get_recon(algs[i]))
        plan.close()
    plans = [mk(i, spec) for i, spec in enumerate(MULTI_SPECS)]
    batch = tg.Batch(plans)
    batch.iterate(algs, 1, prms)
    batch.iterate(algs, 2, prms)
    batch.iterate(algs, 1, prms)
    info = batch.info()
    assert info["multi"]
    per_plan = sum(p.info()["batches"] * 3 for p in plans)
    assert 0 < info["launches"] < per_plan
    for plan, alg, want in zip(plans, algs, singles):
        assert np.array_equal(bits(plan.get_recon(alg)), bits(want))
    batch.close()
    for p in plans:
        p.close()


def test_batch_with_an_ineligible_plan_uses_per_plan_graph():
    plans = [_plan(64, 40, 3, 1, "sirt", slices_per_pass=2, mode="fast", len_storage="u16",
                   delta_index=True, forward_tiles=True),
             _plan(48, 30, 2, 2, "sirt", slices_per_pass=1)]  # exact mode
    batch = tg.Batch(plans)
    batch.iterate("sirt", 2)
    assert not batch.info()["multi"]
    assert batch.info()["launches"] == sum(p.info()["batches"] * (3 if i == 0 else 2)
                                           for i, p in enumerate(plans))
    batch.close()
    for p in plans:
        p.close()


@pytest.mark.parametrize("graphs", [False, True])
@pytest.mark.parametrize("alg", ["sirt", "mlem", "pml", "apmlr"])
def test_two_stream_iterations_match_one_stream(graphs, alg):
    """batch_streams = 2 (odd slice batches on the plan's second stream, with
    their own partial sums and factors) gives the same bits as one stream,
    eagerly and replayed from CUDA graphs; a user stream set on the plan
    still sees the whole iteration in its order."""
    import torch
    prm = tg.default_params(alg, beta=0.3)
    outs = []
    for streams in (1, 2):
        plan = _plan(96, 70, 21, 3, alg, slices_per_pass=4, mode="fast", len_storage="u16",
                     delta_index=True, forward_tiles=True, half_gathers=True,
                     batch_streams=streams)
        user = torch.cuda.Stream()
        plan.set_stream(user.cuda_stream)
        plan.set_graphs(graphs)
        plan.iterate(alg, 3, prm)
        plan.iterate(alg, 2, prm)
        outs.append(plan.get_recon(alg))
        plan.close()
    assert np.array_equal(bits(outs[0]), bits(outs[1]))


@pytest.mark.parametrize("alg", ["sirt", "pml", "apmlr"])
@pytest.mark.parametrize("kind", ["locked", "device", "pageable"])
def test_iterate_with_download_matches_iterate_then_get_recon(alg, kind):
    """tg_iterate_get_recon gives the bits of tg_iterate + tg_get_recon: with
    the last iteration's slice batches written out as each one finishes
    (page-locked or device output; two streams, graphs on, a ragged last
    batch), or one call after the other (APMLR's halo slices, pageable
    output); later iterations continue from the same state."""
    torch = pytest.importorskip("torch")
    C, P, S = 64, 40, 11
    th = theta_uniform(P)
    rng = np.random.default_rng(19)
    sino = rng.uniform(0.5, 2.0, (P, S, C)).astype(np.float32)
    prm = tg.default_params(alg, beta=0.3)
    kw = dict(slices_per_pass=4, mode="fast", len_storage="u16", delta_index=True,
              forward_tiles=True, half_gathers=True)
    halo = 1 if alg == "apmlr" else 0
    shape = (S + 2 * halo, C, C)

    def make():
        plan = tg.Plan(P, S, C, th, **kw)
        plan.set_graphs(True)
        plan.set_sinogram(sino, apply_abs=alg != "sirt")
        plan.reset_recon(alg)
        return plan

    a, b = make(), make()
    a.iterate(alg, 3, prm)
    want = a.get_recon(alg)
    if kind == "locked":
        out = torch.empty(shape, dtype=torch.float32).pin_memory()
    elif kind == "device":
        out = torch.empty(shape, dtype=torch.float32, device="cuda")
    else:
        out = np.empty(shape, np.float32)
    got = b.iterate(alg, 3, prm, out=out)
    b.synchronize()  # device output: ordered on the plan's stream
    got = got.cpu().numpy() if hasattr(got, "cpu") else got
    assert np.array_equal(bits(np.asarray(got)), bits(want))
    a.iterate(alg, 2, prm)
    b.iterate(alg, 2, prm)
    assert np.array_equal(bits(b.get_recon(alg)), bits(a.get_recon(alg)))
    a.close()
    b.close()
