"""trace_gb300: GB300-native iterative reconstruction hot path of Trace.

Python host binding over the C ABI in ``include/trace_gb300.h``. The compute
runs only in the in-tree CUDA library ``trace_gb300/_build/libtrace_gb300.so``;
there is no CPU fallback: importing the bindings without the library raises.

Typical use (mirrors a reference driver's loop, e.g. src/sirt/sirt_main.cc):

    plan = Plan(num_projs=P, num_slices=S, num_cols=C, theta=theta)
    plan.set_sinogram(sino)            # [P][S][C] float32
    plan.reset_recon("sirt")
    plan.iterate("sirt", n_iter=10)
    recon = plan.get_recon("sirt")     # [S][C][C]
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build import LIB as LIB_PATH

ALGS = {"sirt": 0, "mlem": 1, "pml": 2, "apmlr": 3}
LEN_STORAGE = {"f32": 0, "bf16": 1, "f16": 2, "u16": 3}
MODES = {"exact": 0, "fast": 1, "fp64": 2}
STATUS = {0: "OK", 1: "E_ARG", 2: "E_CUDA", 3: "E_NOMEM", 4: "E_STATE",
          5: "E_GEOMETRY", 6: "E_LIMIT"}

EXPORTED = [
    "tg_abi_version", "tg_plan_create", "tg_plan_destroy", "tg_plan_get_info",
    "tg_plan_set_stream", "tg_synchronize", "tg_last_error",
    "tg_degree_to_radian", "tg_set_sinogram", "tg_set_sinogram_clip",
    "tg_reset_recon", "tg_set_recon",
    "tg_get_recon", "tg_reduce", "tg_get_replica", "tg_calculate_fg",
    "tg_get_fg", "tg_update_recon", "tg_reset_replica", "tg_iterate",
    "tg_forward_project", "tg_trace_rays", "tg_plan_set_timing",
    "tg_plan_get_timing", "tg_plan_set_graphs", "tg_batch_create",
    "tg_batch_iterate", "tg_batch_synchronize", "tg_batch_destroy",
    "tg_batch_last_error", "tg_batch_get_info", "tg_host_alloc", "tg_host_free",
    "tg_iterate_get_recon",
]


class TraceError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class PlanDesc(C.Structure):
    _fields_ = [("num_projs", C.c_int), ("num_slices", C.c_int),
                ("num_cols", C.c_int), ("center", C.c_float),
                ("slice_id", C.c_int), ("num_total_slices", C.c_int),
                ("len_storage", C.c_int), ("slices_per_pass", C.c_int),
                ("mode", C.c_int), ("delta_index", C.c_int),
                ("apmlr_fixed_offset", C.c_int), ("forward_tiles", C.c_int),
                ("backward_staged", C.c_int), ("half_gathers", C.c_int),
                ("forward_on_the_fly", C.c_int), ("compensated", C.c_int),
                ("backward_tile_width", C.c_int), ("forward_tile_side", C.c_int),
                ("batch_streams", C.c_int), ("forward_block_warps", C.c_int)]


class Params(C.Structure):
    _fields_ = [("beta", C.c_float), ("beta1", C.c_float), ("delta", C.c_float),
                ("delta1", C.c_float), ("regw", C.c_float)]


class PlanInfo(C.Structure):
    _fields_ = [("num_segments", C.c_int64), ("forward_bytes", C.c_int64),
                ("backward_bytes", C.c_int64), ("device_bytes", C.c_int64),
                ("max_segment_length", C.c_float), ("setup_ms", C.c_double),
                ("batches", C.c_int), ("tile_bytes", C.c_int64),
                ("tile_runs", C.c_int64), ("window_exceptions", C.c_int64),
                ("forward_traced", C.c_int), ("partial_slots", C.c_int64)]


class Timing(C.Structure):
    _fields_ = [("forward_ms", C.c_double), ("backward_ms", C.c_double),
                ("other_ms", C.c_double), ("forward_launches", C.c_int64),
                ("backward_launches", C.c_int64), ("other_launches", C.c_int64)]


_lib = None


def load_library(path: str | None = None) -> C.CDLL:
    """Load the CUDA library (built by ``trace_gb300.build``)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(
            f"trace_gb300 CUDA library not built ({path}); run "
            "`python -m trace_gb300.build` (there is no CPU fallback)")
    lib = C.CDLL(path)
    vp = C.c_void_p
    lib.tg_last_error.restype = C.c_char_p
    lib.tg_last_error.argtypes = [vp]
    lib.tg_plan_create.argtypes = [C.POINTER(PlanDesc), vp, vp, vp, C.POINTER(vp)]
    lib.tg_batch_last_error.restype = C.c_char_p
    lib.tg_batch_last_error.argtypes = [vp]
    lib.tg_host_alloc.argtypes = [C.c_size_t, C.POINTER(vp)]
    lib.tg_host_free.argtypes = [vp]
    for name in EXPORTED:
        getattr(lib, name)  # every declared symbol must exist
    _lib = lib
    return lib


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(C.c_void_p)
    if hasattr(a, "data_ptr"):  # torch tensor (device or host)
        return C.c_void_p(a.data_ptr())
    return C.c_void_p(int(a))


def _is_device(a):
    return hasattr(a, "data_ptr") and getattr(a, "is_cuda", False)


def _host_out(out, shape):
    """A new float32 host array of `shape`, or the caller's host buffer (numpy
    array or CPU tensor; page-locked memory is written by the kernels in
    place) after checking that it is C-contiguous float32 of that shape."""
    if out is None:
        return np.empty(shape, np.float32)
    view = out.numpy() if hasattr(out, "numpy") else out
    if (not isinstance(view, np.ndarray) or view.dtype != np.float32
            or view.shape != tuple(shape) or not view.flags.c_contiguous):
        raise ValueError(f"out must be a C-contiguous float32 array of shape {tuple(shape)}")
    return out


class _HostBlock:
    """Page-locked host memory from tg_host_alloc, freed with the object."""

    def __init__(self, nbytes):
        self._lib = load_library()
        self.ptr = C.c_void_p()
        rc = self._lib.tg_host_alloc(C.c_size_t(nbytes), C.byref(self.ptr))
        if rc:
            raise TraceError(rc, self._lib.tg_last_error(None).decode())

    def __del__(self):
        if getattr(self, "ptr", None) and self.ptr.value:
            self._lib.tg_host_free(self.ptr)
            self.ptr = C.c_void_p()


def host_empty(shape, dtype=np.float32) -> np.ndarray:
    """An uninitialised C-contiguous host array in page-locked memory
    (tg_host_alloc): sinograms uploaded from it and reconstructions, replicas
    and projections downloaded into it are read and written in place by the
    plan's kernels. The memory is freed when the array is."""
    shape = tuple(int(s) for s in np.atleast_1d(shape))
    n = int(np.prod(shape)) * np.dtype(dtype).itemsize
    if n == 0:
        return np.empty(shape, dtype)
    block = _HostBlock(n)
    raw = (C.c_char * n).from_address(block.ptr.value)
    raw._block = block  # the array keeps raw alive, raw keeps the block
    return np.frombuffer(raw, dtype=dtype).reshape(shape)


def default_params(alg: str, beta=None, beta1=1.0, delta=1.0, delta1=1.0,
                   regw=1.0) -> Params:
    """Reference defaults: PML beta 10 (pml_main.cc:20), APMLR beta0=10,
    beta1=1, delta0=1, delta1=1, regw=1 (apmlr_main.cc:22-26)."""
    return Params(10.0 if beta is None else beta, beta1, delta, delta1, regw)


class Plan:
    """One geometry + sinogram + reconstruction on the device."""

    def __init__(self, num_projs, num_slices, num_cols, theta, *, center=0.0,
                 len_storage="f32", slices_per_pass=1, mode="exact",
                 delta_index=False, apmlr_fixed_offset=False, slice_id=0,
                 num_total_slices=None, sin_tab=None, cos_tab=None,
                 forward_tiles=False, backward_staged=False, half_gathers=False,
                 forward_on_the_fly=False, compensated=False, backward_tile_width=0,
                 forward_tile_side=0, batch_streams=0, forward_block_warps=0):
        self._lib = load_library()
        self.P, self.S, self.C = int(num_projs), int(num_slices), int(num_cols)
        d = PlanDesc(self.P, self.S, self.C, float(center), int(slice_id),
                     int(num_total_slices or num_slices),
                     LEN_STORAGE[len_storage] if isinstance(len_storage, str) else int(len_storage),
                     int(slices_per_pass),
                     MODES[mode] if isinstance(mode, str) else int(mode),
                     int(bool(delta_index)), int(bool(apmlr_fixed_offset)),
                     int(bool(forward_tiles)), int(bool(backward_staged)),
                     int(bool(half_gathers)), int(bool(forward_on_the_fly)),
                     int(bool(compensated)), int(backward_tile_width),
                     int(forward_tile_side), int(batch_streams),
                     int(forward_block_warps))
        theta = np.ascontiguousarray(theta, np.float32)
        if theta.size != self.P:
            raise ValueError("theta must have num_projs entries")
        st = ct = None
        if sin_tab is not None:
            st = np.ascontiguousarray(sin_tab, np.float32)
            ct = np.ascontiguousarray(cos_tab, np.float32)
        h = C.c_void_p()
        rc = self._lib.tg_plan_create(C.byref(d), _ptr(theta), _ptr(st), _ptr(ct),
                                      C.byref(h))
        if rc != 0:
            raise TraceError(rc, self._lib.tg_last_error(None).decode())
        self._h = h

    # -- plumbing
    def _chk(self, rc):
        if rc != 0:
            raise TraceError(rc, self._lib.tg_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.tg_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def info(self) -> dict:
        i = PlanInfo()
        self._chk(self._lib.tg_plan_get_info(self._h, C.byref(i)))
        return {f: getattr(i, f) for f, _ in PlanInfo._fields_}

    def set_stream(self, stream_ptr):
        self._chk(self._lib.tg_plan_set_stream(self._h, C.c_void_p(stream_ptr or 0)))

    def set_graphs(self, enable=True):
        """Replay each fused iteration from a captured CUDA graph."""
        self._chk(self._lib.tg_plan_set_graphs(self._h, int(bool(enable))))

    def set_timing(self, enable=True):
        self._chk(self._lib.tg_plan_set_timing(self._h, int(bool(enable))))

    def timing(self) -> dict:
        t = Timing()
        self._chk(self._lib.tg_plan_get_timing(self._h, C.byref(t)))
        return {f: getattr(t, f) for f, _ in Timing._fields_}

    def synchronize(self):
        self._chk(self._lib.tg_synchronize(self._h))

    @staticmethod
    def _alg(alg):
        return ALGS[alg] if isinstance(alg, str) else int(alg)

    def halo(self, alg):
        return 1 if self._alg(alg) == 3 else 0

    # -- data
    def set_sinogram(self, sino, apply_abs=False, clip_min=None):
        """Upload [P][S][C]; apply_abs: |x| (trace_utils::Absolute); clip_min:
        raise values below it to it (after |x|)."""
        dev = _is_device(sino)
        if not dev:
            sino = np.ascontiguousarray(sino, np.float32)
            if sino.shape != (self.P, self.S, self.C):
                raise ValueError(f"sinogram must be [P][S][C] = {(self.P, self.S, self.C)}")
        if clip_min is None:
            self._chk(self._lib.tg_set_sinogram(self._h, _ptr(sino), int(dev),
                                                int(apply_abs)))
        else:
            self._chk(self._lib.tg_set_sinogram_clip(self._h, _ptr(sino), int(dev),
                                                     int(apply_abs), C.c_float(clip_min)))

    def reset_recon(self, alg):
        self._chk(self._lib.tg_reset_recon(self._h, self._alg(alg)))

    def set_recon(self, alg, recon):
        if _is_device(recon):
            self._chk(self._lib.tg_set_recon(self._h, self._alg(alg), _ptr(recon), 1))
            return
        recon = np.ascontiguousarray(recon, np.float32)
        n = self.S + 2 * self.halo(alg)
        if recon.shape != (n, self.C, self.C):
            raise ValueError(f"recon must be {(n, self.C, self.C)}")
        self._chk(self._lib.tg_set_recon(self._h, self._alg(alg), _ptr(recon), 0))

    def get_recon(self, alg, out=None):
        """Download the reconstruction ([S + 2 halo][C][C]) into `out` (a
        device tensor, or a host array / CPU tensor, e.g. pinned, that must be
        float32, C-contiguous and of that shape) or into a new host array."""
        if out is not None and _is_device(out):
            self._chk(self._lib.tg_get_recon(self._h, self._alg(alg), _ptr(out), 1))
            return out
        n = self.S + 2 * self.halo(alg)
        out = _host_out(out, (n, self.C, self.C))
        self._chk(self._lib.tg_get_recon(self._h, self._alg(alg), _ptr(out), 0))
        return out

    # -- operators
    def iterate(self, alg, n_iter=1, params=None, out=None):
        """n_iter fused iterations. With `out` (as for get_recon: a device
        tensor, or a host array / CPU tensor of [S + 2 halo][C][C] float32),
        the reconstruction is also written there and returned, the last
        iteration's slice batches leaving as each one finishes when `out` is
        device or page-locked memory (tg_iterate_get_recon)."""
        p = params if params is not None else default_params(alg)
        if out is None:
            self._chk(self._lib.tg_iterate(self._h, self._alg(alg), C.byref(p), int(n_iter)))
            return None
        if _is_device(out):
            self._chk(self._lib.tg_iterate_get_recon(self._h, self._alg(alg), C.byref(p),
                                                     int(n_iter), _ptr(out), 1))
            return out
        n = self.S + 2 * self.halo(alg)
        out = _host_out(out, (n, self.C, self.C))
        self._chk(self._lib.tg_iterate_get_recon(self._h, self._alg(alg), C.byref(p),
                                                 int(n_iter), _ptr(out), 0))
        return out

    def reduce(self, alg, params=None):
        p = params if params is not None else default_params(alg)
        self._chk(self._lib.tg_reduce(self._h, self._alg(alg), C.byref(p)))

    def get_replica(self, alg, out=None):
        """The reduction replica, [S][2 C C] (per pixel: value, weight), into
        `out` (a host array or CPU tensor of that shape) or a new array."""
        out = _host_out(out, (self.S, 2 * self.C * self.C))
        self._chk(self._lib.tg_get_replica(self._h, self._alg(alg), _ptr(out), 0))
        return out

    def calculate_fg(self, alg, params=None):
        p = params if params is not None else default_params(alg)
        self._chk(self._lib.tg_calculate_fg(self._h, self._alg(alg), C.byref(p)))

    def get_fg(self):
        F = np.empty((self.S, self.C, self.C), np.float32)
        G = np.empty_like(F)
        self._chk(self._lib.tg_get_fg(self._h, _ptr(F), _ptr(G), 0))
        return F, G

    def update_recon(self, alg, params=None):
        p = params if params is not None else default_params(alg)
        self._chk(self._lib.tg_update_recon(self._h, self._alg(alg), C.byref(p)))

    def reset_replica(self):
        self._chk(self._lib.tg_reset_replica(self._h))

    def forward_project(self, alg="sirt", out=None):
        p = default_params(alg)
        if out is not None and _is_device(out):
            self._chk(self._lib.tg_forward_project(self._h, self._alg(alg), C.byref(p), _ptr(out), 1))
            return out
        out = _host_out(out, (self.P, self.S, self.C))
        self._chk(self._lib.tg_forward_project(self._h, self._alg(alg), C.byref(p), _ptr(out), 0))
        return out

    def trace_rays(self, counts_only=False):
        """(counts, offsets, idx, len, len2) of every ray, r = p*C + c;
        counts_only: just the per-ray segment counts."""
        R = self.P * self.C
        counts = np.empty(R, np.int32)
        self._chk(self._lib.tg_trace_rays(self._h, _ptr(counts), None, None, None, None))
        if counts_only:
            return counts
        offs = np.zeros(R + 1, np.int64)
        np.cumsum(counts, out=offs[1:])
        n = int(offs[-1])
        idx = np.empty(n, np.int32)
        ln = np.empty(n, np.float32)
        ln2 = np.empty(n, np.float32)
        self._chk(self._lib.tg_trace_rays(self._h, _ptr(counts), _ptr(offs), _ptr(idx),
                                          _ptr(ln), _ptr(ln2)))
        return counts, offs, idx, ln, ln2


class Batch:
    """Independent plans advanced together, one CUDA graph launch per
    iteration (tg_batch_*)."""

    def __init__(self, plans):
        self._lib = load_library()
        self.plans = list(plans)
        arr = (C.c_void_p * len(self.plans))(*[p.handle for p in self.plans])
        h = C.c_void_p()
        rc = self._lib.tg_batch_create(arr, len(self.plans), C.byref(h))
        if rc:
            raise TraceError(rc, self._lib.tg_batch_last_error(None).decode())
        self._h = h

    def iterate(self, algs, n_iter=1, params=None):
        n = len(self.plans)
        if isinstance(algs, (str, int)):
            algs = [algs] * n
        a = (C.c_int * n)(*[ALGS[x] if isinstance(x, str) else int(x) for x in algs])
        if params is None:
            params = [default_params(x) for x in algs]
        elif isinstance(params, Params):
            params = [params] * n
        pr = (Params * n)(*params)
        rc = self._lib.tg_batch_iterate(self._h, a, pr, int(n_iter))
        if rc:
            raise TraceError(rc, self._lib.tg_batch_last_error(self._h).decode())

    def info(self) -> dict:
        """multi: whether iterations use the multi-plan launches; launches:
        kernel launches per iteration of the last iterate call."""
        m, n = C.c_int(), C.c_int()
        rc = self._lib.tg_batch_get_info(self._h, C.byref(m), C.byref(n))
        if rc:
            raise TraceError(rc, "tg_batch_get_info")
        return {"multi": bool(m.value), "launches": n.value}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.tg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def degree_to_radian(theta):
    t = np.ascontiguousarray(theta, np.float32).copy()
    lib = load_library()
    rc = lib.tg_degree_to_radian(_ptr(t), C.c_int(t.size))
    if rc:
        raise TraceError(rc, "bad theta")
    return t
