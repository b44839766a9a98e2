"""The device tracer (tg::trace_ray in trace_gb300/csrc/tg_device.cuh) finds
each crossing list's first crossing inside the grid by bisection and stops a
cursor at its first crossing outside, relying on the crossings inside being
one contiguous run of line indices (each coordinate is a monotone function
of the line index in IEEE single precision). This checks that property and
the bisection's answer against the reference's full evaluation and trim
(trace_utils.cc:48-111), in float32 as the device computes, over random and
degenerate angles."""
import numpy as np

F = np.float32


def ray_lists(C, s, co, c, mov):
    with np.errstate(all="ignore"):
        xi = F(-1e6)
        yi = F((1 - C) / 2.0 + c + mov)
        srcx = F(F(xi * co) - F(yi * s))
        srcy = F(F(xi * s) + F(yi * co))
        detx = -F(F(xi * co) + F(yi * s))
        dety = F(F(-xi * s) + F(yi * co))
        slope = F(F(srcy - dety) / F(srcx - detx))
        islope = F(F(1.0) / slope)
        gl = (np.arange(C + 1, dtype=np.float32) - F(C / 2.0)).astype(np.float32)
        ax = (F(islope) * (gl - srcy).astype(np.float32)).astype(np.float32) + srcx
        by = (F(slope) * (gl - srcx).astype(np.float32)).astype(np.float32) + srcy
    lo, hi = gl[0], gl[-1]
    return ax.astype(np.float32), by.astype(np.float32), islope, slope, lo, hi


def first_true(n, pred):
    lo, hi = 0, n + 1
    while lo < hi:
        mid = (lo + hi) >> 1
        if pred(mid):
            hi = mid
        else:
            lo = mid + 1
    return lo


def check_list(vals, up, lo, hi):
    """vals in the cursor's order; up: non-decreasing in that order."""
    with np.errstate(invalid="ignore"):
        inside = (vals > lo) & (vals < hi)
    idx = np.flatnonzero(inside)
    if idx.size:  # one contiguous run
        assert idx[-1] - idx[0] + 1 == idx.size
    n = vals.size - 1
    with np.errstate(invalid="ignore"):
        k = first_true(n, lambda k: bool(vals[k] > lo) if up else bool(vals[k] < hi))
    found = k if (k <= n and inside[k]) else None
    want = int(idx[0]) if idx.size else None
    assert found == want


def run_case(C, theta, mov=0.0):
    s, co = F(np.sin(F(theta))), F(np.cos(F(theta)))
    quad = 1 if (0 <= theta % np.pi < np.pi / 2) else 0
    for c in range(C):
        ax, by, islope, slope, lo, hi = ray_lists(C, s, co, c, mov)
        da = 1 if quad else -1
        a_vals = ax if da > 0 else ax[::-1]
        a_up = (not np.signbit(islope)) if da > 0 else bool(np.signbit(islope))
        check_list(a_vals, a_up, lo, hi)
        check_list(by, not np.signbit(slope), lo, hi)


def test_random_angles():
    rng = np.random.default_rng(1)
    for C in (17, 64, 255):
        for theta in rng.uniform(0, 2 * np.pi, 12):
            run_case(C, float(theta), mov=1e-6)


def test_degenerate_angles():
    half_pi = float(np.float32(np.pi / 2))
    for theta in (0.0, 1e-30, 1e-39, 1e-7, half_pi, float(np.nextafter(F(half_pi), F(2))),
                  float(np.nextafter(F(half_pi), F(0))), np.pi, 3 * np.pi / 2):
        run_case(48, theta, mov=1e-6)
