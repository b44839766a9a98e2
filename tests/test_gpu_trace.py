"""GPU tracer parity: pixel-index lists, lengths and squared lengths of every
ray must be bit-identical to the reference (golden fixtures) and to the
oracle on fresh geometries."""
import hashlib

import numpy as np
import pytest

import trace_gb300 as tg
from oracle import oracle as O
from tests._util import bits, golden, tables, theta_uniform

pytestmark = pytest.mark.gpu

FIXTURES = ["trace_c16_p12.npz", "trace_c17_p9.npz", "trace_c24_p7_center.npz",
            "trace_c64_p45.npz", "trace_c256_p180.npz", "trace_c255_p17.npz"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", FIXTURES)
def test_gpu_trace_matches_reference_fixture(name):
    f = golden(name)
    s, c, _ = tables(f)
    plan = tg.Plan(int(f["P"]), 1, int(f["C"]), f["theta"], center=float(f["center"]),
                   sin_tab=s, cos_tab=c)
    counts, offs, idx, ln, ln2 = plan.trace_rays()
    assert np.array_equal(counts, f["counts"])
    assert sha(idx) == str(f["sha_idx"])
    assert sha(ln) == str(f["sha_len"])
    assert sha(ln2) == str(f["sha_len2"])
    assert plan.info()["num_segments"] == int(f["nseg"])
    plan.close()


@pytest.mark.parametrize("C,P,center", [(128, 100, 0.0), (1000, 30, 0.0),
                                        (97, 61, 47.25), (2048, 6, 0.0)])
def test_gpu_trace_matches_oracle_host_tables(C, P, center):
    th = theta_uniform(P)
    tabs = O.angle_table(th)  # this host's sinf/cosf, as the plan computes them
    plan = tg.Plan(P, 1, C, th, center=center)
    g = plan.trace_rays()
    o = O.trace(C, tabs, center)
    assert np.array_equal(g[0], o[0])
    assert np.array_equal(g[2], o[2])
    assert np.array_equal(bits(g[3]), bits(o[3]))
    assert np.array_equal(bits(g[4]), bits(o[4]))
    plan.close()


def test_gpu_trace_arbitrary_angles_full_circle():
    rng = np.random.default_rng(5)
    th = np.concatenate([np.array([0.0, np.pi / 2, np.pi, 3 * np.pi / 2], np.float32),
                         rng.uniform(0, 2 * np.pi, 40).astype(np.float32)])
    tabs = O.angle_table(th)
    plan = tg.Plan(th.size, 1, 64, th)
    g = plan.trace_rays()
    o = O.trace(64, tabs)
    assert np.array_equal(g[2], o[2]) and np.array_equal(bits(g[3]), bits(o[3]))
    plan.close()


@pytest.mark.parametrize("storage", ["f32", "bf16", "f16", "u16"])
@pytest.mark.parametrize("delta", [False, True])
def test_matrix_storage_variants_build(storage, delta):
    th = theta_uniform(90)
    plan = tg.Plan(90, 1, 128, th, len_storage=storage, delta_index=delta)
    info = plan.info()
    assert info["num_segments"] > 0
    assert 1.41 < info["max_segment_length"] < 1.6
    plan.close()


@pytest.mark.parametrize("C", [64, 37])
def test_gpu_trace_degenerate_angles(C):
    """The tracer's bisection for the first crossing inside the grid and its
    stop at the first one outside give the reference's trimmed lists also
    where the slopes are zero, infinite or tiny: exact 0 / 90 degree tables,
    subnormal and tiny angles, one ulp around 90 degrees, negative and
    beyond-2pi angles."""
    half_pi = np.float32(np.pi / 2)
    th = np.array([0.0, 1e-30, 1e-39, 1e-7, half_pi,
                   np.nextafter(half_pi, np.float32(2)), np.nextafter(half_pi, np.float32(0)),
                   np.pi, 3 * np.pi / 2, -0.3, 7.0, 2.5], np.float32)
    s, c, q = O.angle_table(th)
    s, c = s.copy(), c.copy()
    s[4], c[4] = 1.0, 0.0      # exact tables at 90 degrees
    s[7], c[7] = 0.0, -1.0     # and at 180 degrees
    plan = tg.Plan(th.size, 1, C, th, sin_tab=s, cos_tab=c)
    g = plan.trace_rays()
    o = O.trace(C, (s, c, q))
    assert np.array_equal(g[0], o[0])
    assert np.array_equal(g[2], o[2])
    assert np.array_equal(bits(g[3]), bits(o[3]))
    assert np.array_equal(bits(g[4]), bits(o[4]))
    plan.close()
