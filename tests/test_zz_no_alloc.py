"""tg_reduce_slice_noalloc: the reduction entry point for callers that may not
allocate device memory while they run (a host that gives the library a fixed
memory budget up front, or a pipeline that cannot afford the device-wide
synchronisation an allocation may cause). It must give the same replica
numerators as the allocating path (tg_reduce + tg_get_replica) on two calls
in a row, allocate nothing, and refuse geometries beyond its fixed factor
array. Collected last so a stop-at-first-failure run has already run every
other test."""
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


@pytest.mark.parametrize("alg,mode,storage,K", [("sirt", "exact", "f32", 1),
                                                ("pml", "fast", "u16", 4)])
def test_noalloc_matches_allocating_reduce(alg, mode, storage, K):
    torch = pytest.importorskip("torch")
    lib = _lib()
    C_, P, S = 96, 72, 3
    th = theta_uniform(P)
    rng = np.random.default_rng(7)
    sino = rng.uniform(0.5, 2.0, (P, S, C_)).astype(np.float32)
    recon = rng.uniform(0.5, 1.5, (S, C_, C_)).astype(np.float32)
    plan = tg.Plan(P, S, C_, th, slices_per_pass=K, mode=mode, len_storage=storage,
                   delta_index=(storage != "f32"))
    prm = tg.default_params(alg, beta=0.3)
    plan.set_sinogram(sino)
    plan.set_recon(alg, recon)
    plan.reduce(alg, prm)
    want = plan.get_replica(alg)[:, 0::2].reshape(S, C_, C_)

    torch.cuda.synchronize()
    held = plan.info()["device_bytes"]
    outs = []
    for s in (0, 2):  # two calls in a row share the factor array
        r = _dev(recon[s], torch)
        sg = _dev(sino[:, s, :], torch)
        out = torch.full((C_, C_), float("nan"), device="cuda")
        torch.cuda.synchronize()
        rc = lib.tg_reduce_slice_noalloc(plan.handle, tg.ALGS[alg], C.byref(prm),
                                         r.data_ptr(), sg.data_ptr(), out.data_ptr())
        assert rc == 0, lib.tg_last_error(plan.handle)
        plan.synchronize()
        outs.append((s, out.cpu().numpy()))
    assert plan.info()["device_bytes"] == held  # the library allocated nothing
    for s, got in outs:
        assert np.isfinite(got).all()
        assert rel_l2(got, want[s]) < 1e-6, (s, rel_l2(got, want[s]))
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
