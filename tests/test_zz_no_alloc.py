"""tg_reduce_slice_noalloc: the reduction entry point for callers that may not
allocate device memory while they run (a host that gives the library a fixed
memory budget up front, or a pipeline that cannot afford the device-wide
synchronisation an allocation may cause). It must give the same replica
numerators as the allocating path (tg_reduce + tg_get_replica) on two calls
in a row, leave the device's free memory unchanged, and refuse geometries
beyond its fixed factor array. Collected last so a stop-at-first-failure run
has already run every other test."""
import ctypes as C

import numpy as np
import pytest

import trace_gb300 as tg
from tests._util import rel_l2, theta_uniform

pytestmark = pytest.mark.gpu

MAX_RAYS = 4194304


def _lib():
    lib = tg.load_library()
    f = lib.tg_reduce_slice_noalloc
    f.argtypes = [C.c_void_p, C.c_int, C.POINTER(tg.Params), C.c_void_p,
                  C.c_void_p, C.c_void_p]
    return lib


def _dev(a, torch):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


# (alg, plan options, tolerance against tg_reduce). The entry point always
# runs the ray-ordered forward projection (or the on-the-fly tracer) and the
# L1 backprojection with FP32 factors: where tg_reduce takes the same path
# the numerators agree to 1e-6; on tile-staged plans with half gathers its
# forward reads a half-precision reconstruction tile (1e-4), on staged plans
# its backprojection sums through shared memory (1e-6).
CASES = [
    ("sirt", dict(mode="exact", len_storage="f32"), 1e-6),
    ("pml", dict(mode="fast", len_storage="u16", delta_index=True, slices_per_pass=4), 1e-6),
    ("apmlr", dict(mode="fast", len_storage="u16", delta_index=True, slices_per_pass=2), 1e-6),
    ("mlem", dict(mode="fast", len_storage="u16", delta_index=True, slices_per_pass=8,
                  forward_tiles=True, half_gathers=True), 1e-4),
    ("mlem", dict(mode="fast", len_storage="u16", delta_index=True, slices_per_pass=4,
                  forward_on_the_fly=True), 1e-6),
    ("sirt", dict(mode="fast", len_storage="u16", delta_index=True, slices_per_pass=4,
                  forward_tiles=True, backward_staged=True), 1e-6),
]


@pytest.mark.parametrize("alg,kw,tol", CASES,
                         ids=[f"{a}-{i}" for i, (a, _, _) in enumerate(CASES)])
def test_noalloc_matches_allocating_reduce(alg, kw, tol):
    torch = pytest.importorskip("torch")
    lib = _lib()
    C_, P, S = 96, 72, 3
    th = theta_uniform(P)
    rng = np.random.default_rng(7)
    sino = rng.uniform(0.5, 2.0, (P, S, C_)).astype(np.float32)
    halo = 1 if alg == "apmlr" else 0
    recon = rng.uniform(0.5, 1.5, (S + 2 * halo, C_, C_)).astype(np.float32)
    plan = tg.Plan(P, S, C_, th, **kw)
    prm = tg.default_params(alg, beta=0.3)
    plan.set_sinogram(sino, apply_abs=alg != "sirt")
    plan.set_recon(alg, recon)
    plan.reduce(alg, prm)
    want = plan.get_replica(alg)[:, 0::2].reshape(S, C_, C_)
    host_sino = np.abs(sino) if alg != "sirt" else sino

    # APMLR's forward projection of slice s reads the slice one below it
    # (the reference's offset): reconstruction slot s of the halo layout
    calls = [(s, _dev(recon[s], torch), _dev(host_sino[:, s, :], torch),
              torch.full((C_, C_), float("nan"), device="cuda")) for s in (0, 2, 1)]

    def call(s, r, sg, out):
        rc = lib.tg_reduce_slice_noalloc(plan.handle, tg.ALGS[alg], C.byref(prm),
                                         r.data_ptr(), sg.data_ptr(), out.data_ptr())
        assert rc == 0, lib.tg_last_error(plan.handle)

    # a first call at set-up (its kernels' code is loaded on first launch)
    call(*calls[2])
    plan.synchronize()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for c in calls[:2]:  # two calls in a row share the factor array
        call(*c)
    plan.synchronize()
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0, (free0, free1)  # nothing allocated on the device
    for s, _, _, out in calls:
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel_l2(got, want[s]) < tol, (s, rel_l2(got, want[s]))
    plan.close()


def test_noalloc_stray_segment_geometry():
    """A geometry whose traced rays include a stray segment the 4-bit step
    code cannot hold (868 columns x 1129 angles): the plan traces its
    ray-ordered forward on the fly, and so does the entry point."""
    torch = pytest.importorskip("torch")
    lib = _lib()
    C_, P, S = 868, 1129, 1
    th = theta_uniform(P)
    rng = np.random.default_rng(3)
    sino = rng.uniform(0.5, 2.0, (P, S, C_)).astype(np.float32)
    plan = tg.Plan(P, S, C_, th, mode="fast", len_storage="u16", delta_index=True)
    assert plan.info()["forward_traced"] == 1
    prm = tg.default_params("mlem")
    plan.set_sinogram(sino, apply_abs=True)
    plan.reset_recon("mlem")
    plan.reduce("mlem", prm)
    want = plan.get_replica("mlem")[0, 0::2].reshape(C_, C_)
    r = torch.ones((C_, C_), device="cuda")
    sg = _dev(sino[:, 0, :], torch)
    out = torch.full((C_, C_), float("nan"), device="cuda")
    rc = lib.tg_reduce_slice_noalloc(plan.handle, tg.ALGS["mlem"], C.byref(prm),
                                     r.data_ptr(), sg.data_ptr(), out.data_ptr())
    assert rc == 0, lib.tg_last_error(plan.handle)
    plan.synchronize()
    assert rel_l2(out.cpu().numpy(), want) < 1e-6
    plan.close()


def test_noalloc_rejects_geometry_beyond_factor_array():
    torch = pytest.importorskip("torch")
    lib = _lib()
    C_ = 32
    P = MAX_RAYS // C_ + 1  # one angle too many
    plan = tg.Plan(P, 1, C_, theta_uniform(P), len_storage="u16", delta_index=True)
    buf = torch.zeros(P * C_, device="cuda")
    rc = lib.tg_reduce_slice_noalloc(plan.handle, 0, None, buf.data_ptr(),
                                     buf.data_ptr(), buf.data_ptr())
    assert rc == 6  # TG_E_LIMIT
    assert b"4,194,304" in lib.tg_last_error(plan.handle)
    plan.close()


def test_noalloc_null_buffers_rejected():
    lib = _lib()
    plan = tg.Plan(16, 1, 16, theta_uniform(16))
    assert lib.tg_reduce_slice_noalloc(plan.handle, 0, None, None, None, None) == 1
    plan.close()
