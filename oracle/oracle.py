"""Test infrastructure only: Python access to the oracle.

Two checkers live here:
  * the CPU restatement (``trace_oracle.cc`` -> ``_build/liboracle.so``), built
    wherever the tests run, and
  * the reference's own code compiled unmodified (``_ref/libtrace_ref.so``),
    present only where the reference sources are.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
may use this module; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liboracle.so")
# the same port built with -ffast-math (the reference's MLEM/APMLR flags):
# for timing the CPU baseline only
PORT_FAST_SO = os.path.join(HERE, "_build", "liboracle_fastmath.so")
REF_SO = os.path.join(HERE, "_ref", "libtrace_ref.so")
# the reference checkout, given by the environment (no default location)
REF_SRC = os.environ.get("TRACE_REFERENCE_DIR", "")

SIRT, MLEM, PML, APMLR = 0, 1, 2, 3
ALGS = {"sirt": SIRT, "mlem": MLEM, "pml": PML, "apmlr": APMLR}
F32, F64 = 0, 1


def build_port(quiet: bool = True) -> str:
    subprocess.run(["make", "-s", "-j2", "port"], cwd=HERE, check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return PORT_SO


def build_ref(quiet: bool = True) -> str | None:
    """Compile the reference sources named by TRACE_REFERENCE_DIR into _ref/
    (None when the variable is unset or names no reference checkout)."""
    if not REF_SRC or not os.path.isdir(os.path.join(REF_SRC, "src", "common")):
        return None
    subprocess.run(["make", "-s", "-j8", "ref", f"REF={REF_SRC}"], cwd=HERE,
                   check=True, stdout=subprocess.DEVNULL if quiet else None)
    return REF_SO


class _RunArgs(C.Structure):
    _fields_ = [
        ("alg", C.c_int), ("precision", C.c_int), ("dlen", C.c_int),
        ("num_projs", C.c_int), ("num_slices", C.c_int), ("num_cols", C.c_int),
        ("center", C.c_float),
        ("theta", C.c_void_p), ("sinq", C.c_void_p), ("cosq", C.c_void_p),
        ("quad", C.c_void_p), ("sino", C.c_void_p), ("apply_abs", C.c_int),
        ("n_iter", C.c_int), ("threads", C.c_int),
        ("beta", C.c_float), ("beta1", C.c_float), ("delta", C.c_float),
        ("delta1", C.c_float), ("regw", C.c_float),
        ("slice_id", C.c_int), ("num_total_slices", C.c_int),
        ("apmlr_fixed", C.c_int),
        ("recon_in", C.c_void_p), ("recon_out", C.c_void_p),
        ("iters_out", C.c_void_p), ("replica_out", C.c_void_p),
    ]


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


_port = {}
_ref = None


def port(fast_math=False):
    """The oracle library; fast_math: the -ffast-math build (timing only)."""
    if fast_math not in _port:
        path = PORT_FAST_SO if fast_math else PORT_SO
        if not os.path.exists(path):
            build_port()
        lib = C.CDLL(path)
        lib.tor_run.argtypes = [C.POINTER(_RunArgs)]
        lib.tor_last_loop_seconds.restype = C.c_double
        _port[fast_math] = lib
    return _port[fast_math]


def ref():
    """The compiled reference, or None where it cannot be built."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO) and build_ref() is None:
            return None
        _ref = C.CDLL(REF_SO)
    return _ref


def default_center(num_cols: int) -> float:
    return 0.0  # <= 0 selects C/2 + 1, as TraceMetadata does


def angle_table(theta):
    theta = np.ascontiguousarray(theta, np.float32)
    P = theta.size
    s = np.empty(P, np.float32)
    c = np.empty(P, np.float32)
    q = np.empty(P, np.int32)
    port().tor_angle_table(C.c_int(P), _ptr(theta), _ptr(s), _ptr(c), _ptr(q))
    return s, c, q


def geometry(num_cols, center=0.0):
    mov = C.c_float()
    grid = np.empty(num_cols + 1, np.float32)
    port().tor_geometry(C.c_int(num_cols), C.c_float(center), C.byref(mov), _ptr(grid))
    return float(mov.value), grid


def trace(num_cols, tables, center=0.0, threads=8):
    """Oracle segment lists: (counts, offsets, idx, len, len2), ray r = p*C + c."""
    s, c, q = (np.ascontiguousarray(t) for t in tables)
    P = s.size
    counts = np.empty(P * num_cols, np.int32)
    L = port()
    L.tor_trace_counts(C.c_int(num_cols), C.c_int(P), C.c_float(center), _ptr(s),
                       _ptr(c), _ptr(q), _ptr(counts), C.c_int(threads))
    offs = np.zeros(P * num_cols + 1, np.int64)
    np.cumsum(counts, out=offs[1:])
    n = int(offs[-1])
    idx = np.empty(n, np.int32)
    ln = np.empty(n, np.float32)
    ln2 = np.empty(n, np.float32)
    L.tor_trace_fill(C.c_int(num_cols), C.c_int(P), C.c_float(center), _ptr(s),
                     _ptr(c), _ptr(q), _ptr(offs), _ptr(idx), _ptr(ln), _ptr(ln2),
                     C.c_int(threads))
    return counts, offs, idx, ln, ln2


def run(alg, sino, theta=None, tables=None, *, n_iter=1, precision=F32, dlen=0,
        center=0.0, threads=1, beta=10.0, beta1=1.0, delta=1.0, delta1=1.0,
        regw=1.0, slice_id=0, num_total_slices=None, apply_abs=None,
        apmlr_fixed=0, recon_in=None, want_iters=False, want_replica=False,
        fast_math=False):
    """Oracle reconstruction. sino is [P][S][C] float32. fast_math: run the
    -ffast-math build (timing the reference's MLEM/APMLR flags; results are
    not the reference's arithmetic).

    Returns dict(recon, iters, replica, seconds). recon has S + 2*halo
    slices (halo = 1 for APMLR)."""
    if isinstance(alg, str):
        alg = ALGS[alg]
    sino = np.ascontiguousarray(sino, np.float32)
    P, S, Cn = sino.shape
    halo = 1 if alg == APMLR else 0
    dt = np.float32 if precision == F32 else np.float64
    out = np.empty((S + 2 * halo, Cn, Cn), dt)
    iters = np.empty((n_iter, S + 2 * halo, Cn, Cn), dt) if want_iters else None
    rep = np.empty((S, 2 * Cn * Cn), dt) if want_replica else None
    a = _RunArgs()
    a.alg, a.precision, a.dlen = alg, precision, dlen
    a.num_projs, a.num_slices, a.num_cols = P, S, Cn
    a.center = center
    keep = []
    if tables is not None:
        s, c, q = (np.ascontiguousarray(t) for t in tables)
        keep += [s, c, q]
        a.sinq, a.cosq, a.quad = _ptr(s), _ptr(c), _ptr(q)
    else:
        th = np.ascontiguousarray(theta, np.float32)
        keep.append(th)
        a.theta = _ptr(th)
    a.sino = _ptr(sino)
    a.apply_abs = (0 if alg == SIRT else 1) if apply_abs is None else int(apply_abs)
    a.n_iter, a.threads = n_iter, threads
    a.beta, a.beta1, a.delta, a.delta1, a.regw = beta, beta1, delta, delta1, regw
    a.slice_id = slice_id
    a.num_total_slices = S if num_total_slices is None else num_total_slices
    a.apmlr_fixed = apmlr_fixed
    if recon_in is not None:
        recon_in = np.ascontiguousarray(recon_in, dt)
        keep.append(recon_in)
        a.recon_in = _ptr(recon_in)
    a.recon_out, a.iters_out, a.replica_out = _ptr(out), _ptr(iters), _ptr(rep)
    L = port(fast_math)
    rc = L.tor_run(C.byref(a))
    if rc != 0:
        raise ValueError(f"tor_run failed with status {rc}")
    return {"recon": out, "iters": iters, "replica": rep,
            "seconds": L.tor_last_loop_seconds()}


# ---- the compiled reference -------------------------------------------------

def ref_trace(num_cols, theta, center=0.0):
    """Reference segment lists + the per-angle tables it used."""
    L = ref()
    if L is None:
        raise RuntimeError("reference sources unavailable")
    theta = np.ascontiguousarray(theta, np.float32)
    P = theta.size
    counts = np.empty(P * num_cols, np.int32)
    s = np.empty(P, np.float32)
    c = np.empty(P, np.float32)
    q = np.empty(P, np.int32)
    L.ref_trace(C.c_int(num_cols), C.c_int(P), _ptr(theta), C.c_float(center),
                _ptr(counts), None, None, None, None, _ptr(s), _ptr(c), _ptr(q))
    offs = np.zeros(P * num_cols + 1, np.int64)
    np.cumsum(counts, out=offs[1:])
    n = int(offs[-1])
    idx = np.empty(n, np.int32)
    ln = np.empty(n, np.float32)
    ln2 = np.empty(n, np.float32)
    L.ref_trace(C.c_int(num_cols), C.c_int(P), _ptr(theta), C.c_float(center),
                _ptr(counts), _ptr(offs), _ptr(idx), _ptr(ln), _ptr(ln2), None,
                None, None)
    return counts, offs, idx, ln, ln2, (s, c, q)


def ref_run(alg, sino, theta, *, n_iter=1, center=0.0, threads=1, beta=10.0,
            beta1=1.0, delta=1.0, delta1=1.0, regw=1.0, slice_id=0,
            num_total_slices=None, apply_abs=-1, want_iters=False,
            want_replica=False):
    L = ref()
    if L is None:
        raise RuntimeError("reference sources unavailable")
    if isinstance(alg, str):
        alg = ALGS[alg]
    fn = [L.ref_run_sirt, L.ref_run_mlem, L.ref_run_pml, L.ref_run_apmlr][alg]
    sino = np.ascontiguousarray(sino, np.float32)
    P, S, Cn = sino.shape
    halo = 1 if alg == APMLR else 0
    theta = np.ascontiguousarray(theta, np.float32)
    params = np.array([beta, beta1, delta, delta1, regw], np.float32)
    out = np.empty((S + 2 * halo, Cn, Cn), np.float32)
    iters = np.empty((n_iter, S + 2 * halo, Cn, Cn), np.float32) if want_iters else None
    rep = np.empty((S, 2 * Cn * Cn), np.float32) if want_replica else None
    fn(C.c_int(P), C.c_int(S), C.c_int(Cn), _ptr(theta), _ptr(sino),
       C.c_float(center), C.c_int(n_iter), C.c_int(threads), _ptr(params),
       C.c_int(slice_id), C.c_int(S if num_total_slices is None else num_total_slices),
       C.c_int(apply_abs), _ptr(out), _ptr(iters), _ptr(rep))
    return {"recon": out, "iters": iters, "replica": rep}


def forward(recon, tables, center=0.0, threads=8):
    """Sequential-float forward projection: sim [P][S][C] of recon [S][C][C]."""
    recon = np.ascontiguousarray(recon, np.float32)
    S, Cn, _ = recon.shape
    s, c, q = (np.ascontiguousarray(t) for t in tables)
    P = s.size
    sim = np.empty((P, S, Cn), np.float32)
    rc = port().tor_forward(C.c_int(Cn), C.c_int(P), C.c_int(S), C.c_float(center),
                            _ptr(s), _ptr(c), _ptr(q), _ptr(recon), _ptr(sim),
                            C.c_int(threads))
    if rc:
        raise ValueError("tor_forward failed")
    return sim


def fg(alg, recon, W, *, beta=10.0, beta1=1.0, delta=1.0, delta1=1.0, regw=1.0,
       slice_id=0, num_total_slices=None):
    """F and G as CalculateFG leaves them. recon includes APMLR's halo slices."""
    if isinstance(alg, str):
        alg = ALGS[alg]
    recon = np.ascontiguousarray(recon, np.float32)
    halo = 1 if alg == APMLR else 0
    S = recon.shape[0] - 2 * halo
    Cn = recon.shape[1]
    W = np.ascontiguousarray(W, np.float32)
    F = np.empty((S, Cn, Cn), np.float32)
    G = np.empty_like(F)
    rc = port().tor_fg(C.c_int(alg), C.c_int(S), C.c_int(Cn), _ptr(recon), _ptr(W),
                       C.c_float(beta), C.c_float(beta1), C.c_float(delta),
                       C.c_float(delta1), C.c_float(regw), C.c_int(slice_id),
                       C.c_int(S if num_total_slices is None else num_total_slices),
                       _ptr(F), _ptr(G))
    if rc:
        raise ValueError("tor_fg failed")
    return F, G
