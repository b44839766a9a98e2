"""Shared helpers for the tests (fixtures, oracle access, comparisons)."""
import os

import numpy as np

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    with np.load(os.path.join(GOLDEN, name), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def theta_uniform(P):
    return (np.arange(P, dtype=np.float64) * np.pi / P).astype(np.float32)


def tables(f):
    return f["sinq"], f["cosq"], f["quad"]


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def ellipse_sino(C, P, S, seed, tabs=None, center=0.0):
    """Seeded random-ellipse phantoms projected by the oracle's tracer."""
    from trace_gb300.phantom import ellipse_phantoms
    ph = ellipse_phantoms(C, S, seed)
    th = theta_uniform(P)
    if tabs is None:
        tabs = O.angle_table(th)
    sim = O.forward(ph, tabs, center)
    return th, tabs, ph, sim


# SIRT at the first benchmark geometry: 256 x 256 grid, 8 slices, 180 angles
# x 256 columns, 10 iterations; seeded random-ellipse phantoms projected by
# the oracle's projector (bit-identical to the reference's ray sum), Poisson
# counts at I0 = 1e4 converted with -log.
CONFIG1 = dict(C=256, P=180, S=8, n_iter=10, i0=1e4, phantom_seed=101, noise_seed=202)


def config1_data():
    """(theta, angle tables, sinogram [P][S][C]) of the SIRT 256 workload."""
    from trace_gb300.phantom import ellipse_phantoms, poisson_log
    c = CONFIG1
    th = theta_uniform(c["P"])
    tabs = O.angle_table(th)
    ph = ellipse_phantoms(c["C"], c["S"], seed=c["phantom_seed"])
    sim = O.forward(ph, tabs, threads=8)  # each ray summed sequentially
    sino = poisson_log(sim, c["i0"], seed=c["noise_seed"], g=c["C"])
    return th, tabs, sino
