"""The C-ABI library: builds for sm_103a, loads, exports every declared
symbol, validates arguments on the host, and fails loudly without a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import trace_gb300 as tg
from trace_gb300 import build as tgb

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "trace_gb300.h")).read()
    return sorted(set(re.findall(r"\b(tg_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    tgb.build()
    return tg.load_library()


def test_every_declared_symbol_is_exported(lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert set(tg.EXPORTED) <= set(syms)


def test_abi_version(lib):
    assert lib.tg_abi_version() == 1


def test_degree_to_radian_matches_reference_formula(lib):
    deg = np.linspace(0, 359, 181).astype(np.float32)
    got = tg.degree_to_radian(deg)
    kpi = np.float32(3.14159265358979)
    want = ((deg * kpi).astype(np.float64) / 180.0).astype(np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def _desc(**kw):
    d = dict(num_projs=10, num_slices=2, num_cols=16, center=0.0, slice_id=0,
             num_total_slices=2, len_storage=0, slices_per_pass=1, mode=0,
             delta_index=0, apmlr_fixed_offset=0)
    d.update(kw)
    return tg.PlanDesc(**d)


@pytest.mark.parametrize("bad", [dict(num_cols=1), dict(num_projs=0),
                                 dict(slices_per_pass=3), dict(len_storage=9),
                                 dict(mode=5), dict(num_slices=0),
                                 dict(num_cols=32769), dict(num_projs=-1)])
def test_invalid_descriptors_rejected_on_host(lib, bad):
    theta = np.zeros(10, np.float32)
    h = C.c_void_p()
    rc = lib.tg_plan_create(C.byref(_desc(**bad)), theta.ctypes.data_as(C.c_void_p),
                            None, None, C.byref(h))
    assert rc == 1
    assert lib.tg_last_error(None)
    assert not h.value


def test_null_arguments_rejected(lib):
    assert lib.tg_plan_create(None, None, None, None, None) == 1
    assert lib.tg_iterate(None, 0, None, 1) == 1
    assert lib.tg_set_sinogram(None, None, 0, 0) == 1


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU failure path")
def test_plan_creation_fails_loudly_without_gpu(lib):
    with pytest.raises(tg.TraceError) as e:
        tg.Plan(8, 1, 16, np.zeros(8, np.float32))
    assert "CUDA" in str(e.value) or "E_CUDA" in str(e.value)


def test_driver_builds_and_rejects_bad_usage(lib):
    import subprocess
    drv = tgb.build_driver()
    r = subprocess.run([drv], capture_output=True, text=True)
    assert r.returncode == 1 and "need" in r.stderr
    r = subprocess.run([drv, "-r", "sirt", "-f", "/nonexistent", "-t", "/nonexistent",
                        "-o", "/tmp/x", "-P", "4", "-S", "1", "-C", "8"],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open" in r.stderr


def test_driver_checks_npy_inputs(lib, tmp_path):
    """The driver's .npy reader (format 1-3, little-endian float32, C
    order) rejects other dtypes, ranks and shapes before any device work."""
    import subprocess
    drv = tgb.build_driver()
    th = tmp_path / "t.npy"
    np.save(th, np.zeros(4, np.float32))
    cases = [(np.zeros((4, 1, 8), np.float64), [], "float32"),
             (np.zeros((4, 8), np.float32), [], "3-dimensional"),
             (np.zeros((4, 1, 8), np.float32), ["-P", "5"], "does not match"),
             (np.asfortranarray(np.zeros((4, 2, 8), np.float32)), [], "C order")]
    for i, (arr, extra, msg) in enumerate(cases):
        sf = tmp_path / f"s{i}.npy"
        np.save(sf, arr)
        r = subprocess.run([drv, "-r", "sirt", "-f", str(sf), "-t", str(th),
                            "-o", str(tmp_path / "r.npy"), *extra],
                           capture_output=True, text=True)
        assert r.returncode == 1 and msg in r.stderr, (msg, r.stderr)
    r = subprocess.run([drv, "-r", "sirt", "-f", str(tmp_path / "s.f32"), "-t", str(th),
                        "-o", str(tmp_path / "r.npy")], capture_output=True, text=True)
    assert r.returncode == 1


def test_ctypes_structures_match_the_header(tmp_path):
    """The Python binding's ctypes structures have the C header's layout:
    size and every field's offset, as a C compiler lays them out."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"tg_plan_desc": tg.PlanDesc, "tg_params": tg.Params,
               "tg_plan_info": tg.PlanInfo, "tg_timing": tg.Timing}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "trace_gb300.h"',
             'int main(void) {']
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ['  return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    got = {}
    for line in out.split("\n"):
        if line:
            cname, field, val = line.split()
            got[(cname, field)] = int(val)
    for cname, py in structs.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)
