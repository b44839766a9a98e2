"""The oracle (CPU restatement) against the reference's own outputs.

Golden fixtures in tests/golden/ were produced by the reference's code
compiled unmodified (tests/golden/make_golden.py). The oracle must match them
bit for bit with one thread; only then is it trusted as the GPU checker.
"""
import hashlib

import numpy as np
import pytest

from oracle import oracle as O
from tests._util import bits, golden, rel_l2, tables, theta_uniform

TRACE = ["trace_c16_p12.npz", "trace_c17_p9.npz", "trace_c24_p7_center.npz",
         "trace_c64_p45.npz", "trace_c255_p17.npz"]
RECON = ["recon_sirt.npz", "recon_mlem.npz", "recon_pml.npz", "recon_apmlr.npz",
         "recon_apmlr_s1.npz", "recon_pml_odd.npz"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", TRACE)
def test_tracer_matches_reference(name):
    f = golden(name)
    counts, offs, idx, ln, ln2 = O.trace(int(f["C"]), tables(f), float(f["center"]))
    assert np.array_equal(counts, f["counts"])
    assert offs[-1] == f["nseg"]
    assert sha(idx) == str(f["sha_idx"])
    assert sha(ln) == str(f["sha_len"])
    assert sha(ln2) == str(f["sha_len2"])
    if "idx" in f:
        assert np.array_equal(idx, f["idx"])
        assert np.array_equal(bits(ln), bits(f["len"]))


@pytest.mark.parametrize("name", RECON)
def test_reconstruction_matches_reference(name):
    f = golden(name)
    b, b1, d, d1, w = (float(v) for v in f["params"])
    r = O.run(str(f["alg"]), f["sino"], tables=tables(f), n_iter=int(f["n_iter"]),
              center=float(f["center"]), beta=b, beta1=b1, delta=d, delta1=d1,
              regw=w, slice_id=int(f["slice_id"]),
              num_total_slices=int(f["num_total_slices"]),
              want_iters=True, want_replica=True)
    assert np.array_equal(bits(r["iters"]), bits(f["iters"]))
    assert np.array_equal(bits(r["replica"]), bits(f["replica"]))


def test_angle_table_quadrants():
    th = np.array([0.0, 0.5, 1.5707963, 2.0, 3.1415926, 3.5, 4.8, 6.0], np.float32)
    s, c, q = O.angle_table(th)
    kpi = np.float32(3.14159265358979)
    half, three_half = kpi / np.float32(2), (np.float32(3) * kpi) / np.float32(2)
    want = [int((0 <= t < half) or (kpi <= t < three_half)) for t in th]
    assert list(q) == want
    assert q[1] == 1 and q[3] == 0 and q[5] == 1 and q[6] == 0
    assert np.max(np.abs(s - np.sin(th))) < 1e-6


def test_fp64_oracle_close_to_fp32():
    f = golden("recon_mlem.npz")
    r32 = O.run("mlem", f["sino"], tables=tables(f), n_iter=3)
    r64 = O.run("mlem", f["sino"], tables=tables(f), n_iter=3, precision=O.F64)
    r64d = O.run("mlem", f["sino"], tables=tables(f), n_iter=3, precision=O.F64, dlen=1)
    assert r64["recon"].dtype == np.float64
    assert rel_l2(r32["recon"], r64["recon"]) < 1e-5
    assert rel_l2(r64d["recon"], r64["recon"]) < 1e-5


def test_threaded_oracle_matches_single_thread():
    f = golden("recon_pml.npz")
    r1 = O.run("pml", f["sino"], tables=tables(f), n_iter=3, beta=0.5)
    r4 = O.run("pml", f["sino"], tables=tables(f), n_iter=3, beta=0.5, threads=4)
    assert rel_l2(r4["recon"], r1["recon"]) < 1e-5


def test_forward_and_fg_helpers_consistent():
    f = golden("recon_pml.npz")
    S, C = int(f["S"]), int(f["C"])
    prev = f["iters"][-2]
    sim = O.forward(prev, tables(f))
    assert sim.shape == (int(f["P"]), S, C)
    W = f["replica"][0].reshape(-1, 2)[:, 1].reshape(C, C)
    F, G = O.fg("pml", prev, W, beta=0.5)
    num = f["replica"].reshape(S, -1, 2)[:, :, 0].reshape(S, C, C)
    new = (-G + np.sqrt(G * G - 8 * num * F)) / (4 * F)
    assert np.array_equal(bits(new), bits(f["iters"][-1]))


@pytest.mark.skipif(O.ref() is None, reason="the compiled reference (oracle/_ref) is unavailable")
def test_oracle_vs_reference_fresh_random_case():
    rng = np.random.default_rng(99)
    C, P, S = 40, 33, 2
    th = rng.uniform(0, 2 * np.pi, P).astype(np.float32)
    sino = rng.uniform(0.1, 3.0, (P, S, C)).astype(np.float32)
    counts, offs, idx, ln, ln2, tabs = O.ref_trace(C, th)
    c2, o2, i2, l2, l22 = O.trace(C, tabs)
    assert np.array_equal(idx, i2) and np.array_equal(bits(ln), bits(l2))
    for alg in ["sirt", "mlem", "pml", "apmlr"]:
        r = O.ref_run(alg, sino, th, n_iter=2, beta=1.5)
        m = O.run(alg, sino, tables=tabs, n_iter=2, beta=1.5)
        assert np.array_equal(bits(r["recon"]), bits(m["recon"])), alg


def test_oracle_pinned_at_sirt256_workload():
    """The oracle reproduces the compiled reference bit for bit at the
    SIRT 256 x 256, 180-angle, 8-slice, 10-iteration workload with Poisson
    data (tests/golden/config1_sirt256.json, made by make_golden.py)."""
    import hashlib
    import json
    import os

    from tests._util import GOLDEN, config1_data
    with open(os.path.join(GOLDEN, "config1_sirt256.json")) as f:
        g = json.load(f)

    def sha(a):
        return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()

    _, tabs, sino = config1_data()
    assert sha(sino) == g["sha_sino"], "input generator changed"
    r = O.run("sirt", sino, tables=tabs, n_iter=g["n_iter"], threads=1, want_iters=True)
    assert [sha(r["iters"][i]) for i in range(g["n_iter"])] == g["sha_iters"]
