"""The tile build splits a cell index into column and row without an integer
division (tg::cell_xy in trace_gb300/csrc/tg_device.cuh): a float quotient
estimate, truncated, then corrected by one from the remainder. This checks,
in IEEE single precision as the device computes it, that one correction
always suffices and gives exact results for every grid size the library
accepts (exhaustively for small grids, sampled up to 32768)."""
import numpy as np


def cell_xy(idx, g):
    idx = np.asarray(idx, np.int64)
    inv_g = np.float32(1.0) / np.float32(g)                     # 1.0f / (float)g
    est = np.float32(idx.astype(np.float32)) * inv_g            # __fmul_rn(__int2float_rn)
    q = np.trunc(est).astype(np.int64)                          # __float2int_rz
    rem = idx - q * g
    low, high = rem < 0, rem >= g
    q = q - low + high
    rem = rem + g * low - g * high
    return rem, q, est


def test_exhaustive_small_grids():
    for g in range(2, 260):
        idx = np.arange(g * g)
        ix, iy, _ = cell_xy(idx, g)
        assert np.array_equal(ix, idx % g) and np.array_equal(iy, idx // g), g


def test_sampled_large_grids():
    rng = np.random.default_rng(0)
    for g in [511, 512, 1000, 1023, 1024, 1536, 2047, 2048, 2049, 4095, 4096, 8191,
              16384, 30001, 32767, 32768]:
        n = g * g
        idx = np.concatenate([rng.integers(0, n, 200_000), np.arange(0, n, g),
                              np.arange(g - 1, n, g), [0, n - 1]])
        ix, iy, est = cell_xy(idx, g)
        assert np.array_equal(ix, idx % g) and np.array_equal(iy, idx // g), g
        # the estimate is within one of the true quotient
        assert np.all(np.abs(est.astype(np.float64) - idx / g) < 1.0), g
