"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference's own tracer, operators and DISP engine, compiled
unmodified from the reference tree by ``oracle/Makefile`` (target ``ref``)
with one reduction thread (the only bit-reproducible setting of its engine).
Needs the reference sources: TRACE_REFERENCE_DIR names the checkout; the
fixtures it writes are what the tests use everywhere else.

    TRACE_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from oracle import oracle as O  # noqa: E402


def theta_uniform(P):
    """theta_k = k*pi/P (radians), computed in double, stored as float."""
    return (np.arange(P, dtype=np.float64) * np.pi / P).astype(np.float32)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def trace_fixture(name, C, P, center=0.0, full=True):
    theta = theta_uniform(P)
    counts, offs, idx, ln, ln2, (s, c, q) = O.ref_trace(C, theta, center)
    d = dict(C=C, P=P, center=np.float32(center), theta=theta, sinq=s, cosq=c,
             quad=q, counts=counts, nseg=np.int64(offs[-1]),
             sha_idx=sha(idx), sha_len=sha(ln), sha_len2=sha(ln2))
    if full:
        d.update(idx=idx, len=ln, len2=ln2)
    np.savez_compressed(os.path.join(HERE, name), **d)
    print(name, "segments", int(offs[-1]))


def recon_fixture(name, alg, C, P, S, n_iter, seed, center=0.0, **params):
    theta = theta_uniform(P)
    rng = np.random.default_rng(seed)
    sino = rng.uniform(0.5, 2.0, size=(P, S, C)).astype(np.float32)
    _, _, _, _, _, (s, c, q) = O.ref_trace(C, theta, center)
    r = O.ref_run(alg, sino, theta, n_iter=n_iter, center=center,
                  want_iters=True, want_replica=True, **params)
    np.savez_compressed(
        os.path.join(HERE, name), alg=alg, C=C, P=P, S=S, n_iter=n_iter,
        center=np.float32(center), theta=theta, sinq=s, cosq=c, quad=q,
        sino=sino, iters=r["iters"], replica=r["replica"],
        params=np.array([params.get(k, d) for k, d in
                         [("beta", 10.0), ("beta1", 1.0), ("delta", 1.0),
                          ("delta1", 1.0), ("regw", 1.0)]], np.float32),
        slice_id=params.get("slice_id", 0),
        num_total_slices=params.get("num_total_slices", S))
    print(name, alg, "ok")


def config1_fixture(name):
    """Hashes of the reference's SIRT run at the 256 x 256, 180-angle,
    8-slice, 10-iteration workload with Poisson data (the input is rebuilt by
    tests._util.config1_data; its hash is stored to catch generator drift)."""
    import json
    from tests._util import CONFIG1, config1_data
    th, _, sino = config1_data()
    r = O.ref_run("sirt", sino, th, n_iter=CONFIG1["n_iter"], want_iters=True)
    d = dict(CONFIG1, sha_sino=sha(sino),
             sha_iters=[sha(r["iters"][i]) for i in range(CONFIG1["n_iter"])],
             norm_iters=[float(np.linalg.norm(r["iters"][i].astype(np.float64)))
                         for i in range(CONFIG1["n_iter"])])
    with open(os.path.join(HERE, name), "w") as f:
        json.dump(d, f, indent=1)
    print(name, "ok")


def main():
    if O.build_ref() is None:
        raise SystemExit("reference sources not available")
    trace_fixture("trace_c16_p12.npz", 16, 12)
    trace_fixture("trace_c17_p9.npz", 17, 9)
    trace_fixture("trace_c24_p7_center.npz", 24, 7, center=11.3)
    trace_fixture("trace_c64_p45.npz", 64, 45, full=False)
    trace_fixture("trace_c256_p180.npz", 256, 180, full=False)
    trace_fixture("trace_c255_p17.npz", 255, 17, full=False)
    recon_fixture("recon_sirt.npz", "sirt", 32, 24, 3, 3, seed=11)
    recon_fixture("recon_mlem.npz", "mlem", 32, 24, 3, 3, seed=12)
    recon_fixture("recon_pml.npz", "pml", 32, 24, 3, 3, seed=13, beta=0.5)
    recon_fixture("recon_apmlr.npz", "apmlr", 32, 24, 3, 3, seed=14, beta=0.5,
                  beta1=0.7, delta=0.8, delta1=1.3, regw=0.9)
    recon_fixture("recon_apmlr_s1.npz", "apmlr", 20, 16, 1, 2, seed=15)
    recon_fixture("recon_pml_odd.npz", "pml", 21, 13, 2, 2, seed=16, beta=2.0,
                  center=9.7)
    config1_fixture("config1_sirt256.json")


if __name__ == "__main__":
    main()
