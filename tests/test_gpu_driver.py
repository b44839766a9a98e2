"""The C++ drop-in classes (trace_gb300/host/trace_gb300.hpp) driven by the
reference drivers' loop (trace_gb300/host/trace_recon.cc), end to end from
raw files, against the oracle on the same host."""
import os
import subprocess

import numpy as np
import pytest

import trace_gb300 as tg
from oracle import oracle as O
from tests._util import rel_l2, theta_uniform
from trace_gb300 import build as tgb

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("alg,extra,params", [
    ("sirt", [], {}),
    ("mlem", ["--fused"], {}),
    ("pml", [], {"beta": 0.4}),
    ("apmlr", [], {"beta": 0.4, "beta1": 0.6, "delta": 0.9, "delta1": 1.1, "regw": 0.8}),
    ("pml", ["--fused", "--len", "u16", "--slices-per-pass", "4", "--fast",
             "--delta-index"], {"beta": 0.4}),
    # the operator loop (Reduce / CalculateFG / UpdateRecon) on tile-ordered plans
    ("pml", ["--len", "u16", "--slices-per-pass", "4", "--fast", "--delta-index",
             "--tiles"], {"beta": 0.4}),
    ("mlem", ["--len", "u16", "--slices-per-pass", "4", "--fast", "--delta-index",
              "--tiles", "--half"], {}),
])
def test_driver_matches_oracle(tmp_path, alg, extra, params):
    tgb.build()
    drv = tgb.build_driver()
    C, P, S, n = 48, 40, 3, 3
    th = theta_uniform(P)
    rng = np.random.default_rng(11)
    sino = rng.uniform(0.5, 2.0, (P, S, C)).astype(np.float32)
    sf, tf, of = tmp_path / "s.f32", tmp_path / "t.f32", tmp_path / "r.f32"
    sino.tofile(sf)
    th.tofile(tf)
    flags = {"beta": "-j", "beta1": "-k", "delta": "-l", "delta1": "-m", "regw": "-w"}
    cmd = [drv, "-r", alg, "-f", str(sf), "-t", str(tf), "-o", str(of), "-P", str(P),
           "-S", str(S), "-C", str(C), "-i", str(n)]
    for k, v in params.items():
        cmd += [flags[k], str(v)]
    r = subprocess.run(cmd + extra, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    halo = 1 if alg == "apmlr" else 0
    got = np.fromfile(of, np.float32).reshape(S + 2 * halo, C, C)
    want = O.run(alg, sino, theta=th, n_iter=n, **params)["recon"]
    tol = 1e-4 if "--fast" in extra else 2e-6
    assert rel_l2(got, want) < tol


@pytest.mark.parametrize("alg", ["sirt", "apmlr"])
def test_driver_npy_files(tmp_path, alg):
    """NumPy files in and out: the shapes come from the sinogram, theta is
    given in degrees (--degrees), and the result matches the oracle."""
    tgb.build()
    drv = tgb.build_driver()
    C, P, S, n = 40, 36, 2, 2
    th = theta_uniform(P)
    deg = (th.astype(np.float64) * 180.0 / np.pi).astype(np.float32)
    rng = np.random.default_rng(5)
    sino = rng.uniform(0.5, 2.0, (P, S, C)).astype(np.float32)
    np.save(tmp_path / "s.npy", sino)
    np.save(tmp_path / "t.npy", deg)
    r = subprocess.run([drv, "-r", alg, "-f", str(tmp_path / "s.npy"), "-t",
                        str(tmp_path / "t.npy"), "-o", str(tmp_path / "r.npy"),
                        "-i", str(n), "--degrees", "-j", "0.4"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.load(tmp_path / "r.npy")
    halo = 1 if alg == "apmlr" else 0
    assert got.shape == (S + 2 * halo, C, C) and got.dtype == np.float32
    rad = tg.degree_to_radian(deg)
    kw = {"beta": 0.4} if alg == "apmlr" else {}
    want = O.run(alg, sino, theta=rad, n_iter=n, **kw)["recon"]
    assert rel_l2(got, want) < 2e-6
