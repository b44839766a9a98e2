"""GPU reconstruction parity against the reference (golden fixtures) and the
oracle.

Tolerances:
  * exact mode, f32 lengths: forward projections bit-identical; F bit-identical;
    reconstructions within 2e-6 relative L2 of the reference per iteration
    (the backprojection adds the two lengths of a ray that re-enters a pixel
    before multiplying, a reassociation the reference does not make);
  * fast mode and 16-bit lengths: relative L2 <= 1e-4 against the FP64 oracle.
"""
import numpy as np
import pytest

import trace_gb300 as tg
from oracle import oracle as O
from tests._util import bits, golden, rel_l2, tables, theta_uniform

pytestmark = pytest.mark.gpu

RECON = ["recon_sirt.npz", "recon_mlem.npz", "recon_pml.npz", "recon_apmlr.npz",
         "recon_apmlr_s1.npz", "recon_pml_odd.npz"]


def params_of(f):
    return tg.Params(*(float(v) for v in f["params"]))


def plan_for(f, **kw):
    s, c, _ = tables(f)
    return tg.Plan(int(f["P"]), int(f["S"]), int(f["C"]), f["theta"],
                   center=float(f["center"]), sin_tab=s, cos_tab=c,
                   slice_id=int(f["slice_id"]),
                   num_total_slices=int(f["num_total_slices"]), **kw)


def load(plan, f):
    alg = str(f["alg"])
    plan.set_sinogram(f["sino"], apply_abs=alg != "sirt")
    plan.reset_recon(alg)
    return alg


@pytest.mark.parametrize("name", RECON)
@pytest.mark.parametrize("K", [1, 2, 4])
def test_exact_iterations_match_reference(name, K):
    f = golden(name)
    plan = plan_for(f, slices_per_pass=K)
    alg = load(plan, f)
    for it in range(int(f["n_iter"])):
        plan.iterate(alg, 1, params_of(f))
        got = plan.get_recon(alg)
        want = f["iters"][it]
        assert rel_l2(got, want) < 2e-6, (name, it)
    plan.close()


@pytest.mark.parametrize("name", ["recon_sirt.npz", "recon_pml.npz", "recon_apmlr.npz"])
def test_batching_is_bit_identical_in_exact_mode(name):
    f = golden(name)
    outs = []
    for K in (1, 2, 4, 8, 16):
        plan = plan_for(f, slices_per_pass=K)
        alg = load(plan, f)
        plan.iterate(alg, int(f["n_iter"]), params_of(f))
        outs.append(plan.get_recon(alg))
        plan.close()
    for o in outs[1:]:
        assert np.array_equal(bits(o), bits(outs[0]))


def test_forward_projection_bit_identical():
    C, P, S = 48, 37, 3
    th = theta_uniform(P)
    tabs = O.angle_table(th)
    rng = np.random.default_rng(3)
    recon = rng.uniform(0, 2, (S, C, C)).astype(np.float32)
    for K in (1, 4):
        plan = tg.Plan(P, S, C, th, slices_per_pass=K)
        plan.set_recon("sirt", recon)
        sim = plan.forward_project("sirt")
        want = O.forward(recon, tabs)
        assert np.array_equal(bits(sim), bits(want))
        plan.close()


@pytest.mark.parametrize("name", ["recon_sirt.npz", "recon_mlem.npz", "recon_pml.npz",
                                  "recon_apmlr.npz"])
def test_operator_sequence_replica_fg_update(name):
    """reduce -> replica, CalculateFG -> F/G, UpdateRecon, as the drivers call them."""
    f = golden(name)
    plan = plan_for(f)
    alg = load(plan, f)
    prm = params_of(f)
    n = int(f["n_iter"])
    halo = 1 if alg == "apmlr" else 0
    if n > 1:
        plan.set_recon(alg, f["iters"][n - 2])
    plan.reduce(alg, prm)
    rep = plan.get_replica(alg)
    want = f["replica"]
    assert rel_l2(rep[:, 1::2], want[:, 1::2]) < 1e-6  # total lengths
    assert rel_l2(rep[:, 0::2], want[:, 0::2]) < 2e-6  # numerators
    if alg in ("pml", "apmlr"):
        plan.calculate_fg(alg, prm)
        F, G = plan.get_fg()
        C = int(f["C"])
        prev = f["iters"][n - 2] if n > 1 else None
        W = rep[0, 1::2].reshape(C, C)
        b, b1, d, d1, w = (float(v) for v in f["params"])
        Fo, Go = O.fg(alg, prev, W, beta=b, beta1=b1, delta=d, delta1=d1, regw=w,
                      slice_id=int(f["slice_id"]),
                      num_total_slices=int(f["num_total_slices"]))
        assert np.array_equal(bits(F), bits(Fo))
        assert np.array_equal(bits(G), bits(Go))
    plan.update_recon(alg, prm)
    got = plan.get_recon(alg)
    assert rel_l2(got, f["iters"][n - 1]) < 2e-6
    # the fused path from the same start agrees with the operator path
    if n > 1:
        plan.set_recon(alg, f["iters"][n - 2])
    else:
        plan.reset_recon(alg)
    plan.iterate(alg, 1, prm)
    assert rel_l2(plan.get_recon(alg), got) < 1e-6
    assert got.shape[0] == int(f["S"]) + 2 * halo
    plan.close()


@pytest.mark.parametrize("alg", ["sirt", "mlem", "pml", "apmlr"])
@pytest.mark.parametrize("storage,mode,delta", [("f32", "fast", False),
                                                ("u16", "fast", True),
                                                ("f16", "fast", True),
                                                ("u16", "exact", False)])
def test_mixed_precision_within_tolerance_of_fp64(alg, storage, mode, delta):
    C, P, S, n_iter = 96, 72, 3, 8
    th = theta_uniform(P)
    tabs = O.angle_table(th)
    from trace_gb300.phantom import ellipse_phantoms
    ph = ellipse_phantoms(C, S, seed=21)
    sino = O.forward(ph, tabs)
    kw = dict(beta=0.05) if alg == "pml" else dict(beta=0.02) if alg == "apmlr" else {}
    ref64 = O.run(alg, sino, tables=tabs, n_iter=n_iter, precision=O.F64, **kw)
    plan = tg.Plan(P, S, C, th, len_storage=storage, mode=mode, delta_index=delta,
                   slices_per_pass=4)
    plan.set_sinogram(sino, apply_abs=alg != "sirt")
    plan.reset_recon(alg)
    plan.iterate(alg, n_iter, tg.default_params(alg, **kw))
    got = plan.get_recon(alg)
    err = rel_l2(got, ref64["recon"])
    assert err < 1e-4, err
    plan.close()


def test_apmlr_fixed_offset_matches_oracle():
    f = golden("recon_apmlr.npz")
    for K in (1, 2):
        plan = plan_for(f, slices_per_pass=K, apmlr_fixed_offset=True)
        alg = load(plan, f)
        b, b1, d, d1, w = (float(v) for v in f["params"])
        plan.iterate(alg, 3, params_of(f))
        o = O.run("apmlr", f["sino"], tables=tables(f), n_iter=3, beta=b, beta1=b1,
                  delta=d, delta1=d1, regw=w, apmlr_fixed=1)
        assert rel_l2(plan.get_recon(alg), o["recon"]) < 2e-6
        plan.close()


def test_slices_not_multiple_of_batch():
    C, P, S = 40, 30, 5
    th = theta_uniform(P)
    tabs = O.angle_table(th)
    rng = np.random.default_rng(8)
    sino = rng.uniform(0.5, 2, (P, S, C)).astype(np.float32)
    o = O.run("mlem", sino, tables=tabs, n_iter=2)
    for K in (2, 4, 8):
        plan = tg.Plan(P, S, C, th, slices_per_pass=K)
        plan.set_sinogram(sino, apply_abs=True)
        plan.reset_recon("mlem")
        plan.iterate("mlem", 2)
        assert rel_l2(plan.get_recon("mlem"), o["recon"]) < 2e-6
        plan.close()


def test_state_errors_are_reported():
    th = theta_uniform(10)
    plan = tg.Plan(10, 2, 16, th)
    with pytest.raises(tg.TraceError) as e:
        plan.iterate("sirt", 1)
    assert e.value.status == 4  # no reconstruction layout yet
    plan.reset_recon("sirt")
    with pytest.raises(tg.TraceError) as e:
        plan.iterate("sirt", 1)
    assert e.value.status == 4  # no sinogram
    with pytest.raises(tg.TraceError) as e:
        plan.iterate("apmlr", 1)
    assert e.value.status == 4  # layout of another family
    with pytest.raises(ValueError):
        plan.set_sinogram(np.zeros((3, 3, 3), np.float32))
    plan.close()


@pytest.mark.parametrize("on_device", [False, True])
def test_sinogram_clip_matches_oracle_on_clipped_input(on_device):
    """tg_set_sinogram_clip: |x| then a floor of 1e-6 (the MLEM workload's
    clip before the ratio step) equals the oracle run on the same sinogram
    with the floor applied on the host."""
    C, P, S = 64, 40, 3
    th = theta_uniform(P)
    tabs = O.angle_table(th)
    from trace_gb300.phantom import ellipse_phantoms
    sino = O.forward(ellipse_phantoms(C, S, seed=11), tabs)
    rng = np.random.default_rng(11)
    mask = rng.uniform(size=sino.shape) < 0.05
    sino[mask] = rng.choice([0.0, -1e-8, 3e-7, -2.0], size=int(mask.sum()))
    floor = np.float32(1e-6)
    host = np.maximum(np.abs(sino), floor).astype(np.float32)
    ref = O.run("mlem", host, tables=tabs, n_iter=4, apply_abs=False)["recon"]
    plan = tg.Plan(P, S, C, th)
    if on_device:
        import torch
        plan.set_sinogram(torch.from_numpy(sino).cuda(), apply_abs=True, clip_min=1e-6)
    else:
        plan.set_sinogram(sino, apply_abs=True, clip_min=1e-6)
    plan.reset_recon("mlem")
    plan.iterate("mlem", 4)
    assert rel_l2(plan.get_recon("mlem"), ref) < 2e-6
    plan.close()


def test_get_recon_into_host_buffers():
    """get_recon writes into a caller's host buffer (numpy or pinned CPU
    tensor) with the same bits as a fresh download, and rejects a buffer of
    the wrong shape or type."""
    torch = pytest.importorskip("torch")
    f = golden("recon_apmlr.npz")
    plan = plan_for(f, slices_per_pass=2)
    alg = load(plan, f)
    plan.iterate(alg, 2, params_of(f))
    want = plan.get_recon(alg)
    host = np.empty_like(want)
    assert plan.get_recon(alg, out=host) is host
    pinned = torch.empty(want.shape, dtype=torch.float32).pin_memory()
    plan.get_recon(alg, out=pinned)
    assert np.array_equal(bits(host), bits(want))
    assert np.array_equal(bits(pinned.numpy()), bits(want))
    with pytest.raises(ValueError):
        plan.get_recon(alg, out=np.empty(want.shape[1:], np.float32))
    with pytest.raises(ValueError):
        plan.get_recon(alg, out=np.empty(want.shape, np.float64))
    plan.close()


def test_page_locked_transfers_match_staged():
    """Page-locked host buffers are read and written by the layout kernels in
    place (no device staging copy): sinogram and reconstruction uploads,
    reconstruction, replica and forward-projection downloads give the same
    bits as pageable and device buffers, also for a buffer that starts
    inside a page-locked block."""
    torch = pytest.importorskip("torch")
    f = golden("recon_pml.npz")
    alg, prm = str(f["alg"]), params_of(f)
    sino = np.ascontiguousarray(f["sino"], np.float32)

    def locked(a, offset=5):
        blk = torch.empty(a.size + offset, dtype=torch.float32).pin_memory()
        view = blk[offset:].view(a.shape)
        view.copy_(torch.from_numpy(np.ascontiguousarray(a)))
        return view

    def run(kind):
        plan = plan_for(f, slices_per_pass=2)
        src = {"pageable": sino, "locked": locked(sino),
               "device": torch.from_numpy(sino).cuda()}[kind]
        plan.set_sinogram(src, apply_abs=True)
        plan.reset_recon(alg)
        plan.iterate(alg, 2, prm)
        return plan

    plans = {k: run(k) for k in ("pageable", "locked", "device")}
    # the page-locked plan has staged nothing (no staging buffer allocated),
    # also after a download into page-locked memory; the pageable one has
    held = plans["locked"].info()["device_bytes"]
    out0 = torch.empty(plans["pageable"].get_recon(alg).shape, dtype=torch.float32).pin_memory()
    plans["locked"].get_recon(alg, out=out0)
    assert plans["locked"].info()["device_bytes"] == held
    assert plans["pageable"].info()["device_bytes"] > held
    want = plans["pageable"].get_recon(alg)
    for k, plan in plans.items():
        assert np.array_equal(bits(plan.get_recon(alg)), bits(want)), k
        out = locked(np.zeros_like(want), offset=3)
        plan.get_recon(alg, out=out)
        assert np.array_equal(bits(out.numpy()), bits(want)), k
    plan = plans["pageable"]
    sim = plan.forward_project(alg)
    sim_locked = locked(np.zeros_like(sim))
    plan.forward_project(alg, out=sim_locked)
    assert np.array_equal(bits(sim_locked.numpy()), bits(sim))
    plan.reset_replica()
    plan.reduce(alg, prm)
    rep = plan.get_replica(alg)
    rep_locked = locked(np.zeros_like(rep))
    plan.get_replica(alg, out=rep_locked)
    assert np.array_equal(bits(rep_locked.numpy()), bits(rep))
    # a reconstruction set from page-locked memory iterates like one set
    # from pageable memory
    start = np.ascontiguousarray(want * 1.5 + 0.25, np.float32)
    for src in (start, locked(start)):
        plan.set_recon(alg, src)
        assert np.array_equal(bits(plan.get_recon(alg)), bits(start))
        plan.iterate(alg, 1, prm)
    a = plan.get_recon(alg)
    plan.set_recon(alg, start)
    plan.iterate(alg, 1, prm)
    assert np.array_equal(bits(plan.get_recon(alg)), bits(a))
    for plan in plans.values():
        plan.close()


def test_host_empty_buffers_are_used_in_place():
    """tg.host_empty (tg_host_alloc) gives page-locked arrays: an upload from
    and a download into them allocate no staging buffer, with the same bits
    as ordinary arrays."""
    f = golden("recon_mlem.npz")
    alg = str(f["alg"])
    sino = tg.host_empty(f["sino"].shape)
    sino[...] = f["sino"]
    outs = []
    for src in (np.array(f["sino"], np.float32), sino):
        plan = plan_for(f)
        plan.set_sinogram(src, apply_abs=True)
        plan.reset_recon(alg)
        plan.iterate(alg, 2, params_of(f))
        held = plan.info()["device_bytes"]
        out = tg.host_empty((int(f["S"]), int(f["C"]), int(f["C"])))
        plan.get_recon(alg, out=out)
        if src is sino:
            assert plan.info()["device_bytes"] == held
        outs.append(np.array(out))
        plan.close()
    assert np.array_equal(bits(outs[0]), bits(outs[1]))
    del sino, out  # freed with the arrays (tg_host_free)


@pytest.mark.parametrize("P", [1920, 1921, 2003])
def test_many_angles(P):
    """Angle counts past several 512-angle chunks of the backprojection's
    staged window coefficients (and not a multiple of 4): against the oracle
    (exact mode) and FP64 (fast mode with half gathers)."""
    C, S, it = 32, 2, 2
    th = theta_uniform(P)
    tabs = O.angle_table(th)
    rng = np.random.default_rng(P)
    sino = rng.uniform(0.5, 2.0, (P, S, C)).astype(np.float32)
    want = O.run("mlem", sino, tables=tabs, n_iter=it)["recon"]
    plan = tg.Plan(P, S, C, th, sin_tab=tabs[0], cos_tab=tabs[1])
    plan.set_sinogram(sino, apply_abs=True)
    plan.reset_recon("mlem")
    plan.iterate("mlem", it)
    assert rel_l2(plan.get_recon("mlem"), want) < 2e-6
    plan.close()
    ref = O.run("mlem", sino, tables=tabs, n_iter=it, precision=O.F64)["recon"]
    plan = tg.Plan(P, S, C, th, sin_tab=tabs[0], cos_tab=tabs[1], slices_per_pass=2,
                   mode="fast", len_storage="u16", delta_index=True, forward_tiles=True,
                   half_gathers=True)
    plan.set_sinogram(sino, apply_abs=True)
    plan.reset_recon("mlem")
    plan.iterate("mlem", it)
    assert rel_l2(plan.get_recon("mlem"), ref) < 1e-4
    plan.close()
