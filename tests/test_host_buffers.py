"""Host-buffer handling of the Python binding, on the CPU: output buffers are
checked before any call reaches the library, and page-locked allocation
fails loudly where there is no GPU."""
import numpy as np
import pytest

import trace_gb300 as tg


def test_host_out_checks_shape_dtype_and_layout():
    shape = (2, 3, 3)
    assert tg._host_out(None, shape).shape == shape
    good = np.zeros(shape, np.float32)
    assert tg._host_out(good, shape) is good
    for bad in (np.zeros((2, 3), np.float32), np.zeros(shape, np.float64),
                np.zeros((2, 3, 6), np.float32)[:, :, ::2], [[0.0]]):
        with pytest.raises(ValueError):
            tg._host_out(bad, shape)


def test_host_empty_without_a_gpu():
    assert tg.host_empty((0, 4)).shape == (0, 4)
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        a = tg.host_empty((4, 5))
        assert a.shape == (4, 5) and a.dtype == np.float32 and a.flags.c_contiguous
        return
    with pytest.raises(tg.TraceError) as e:
        tg.host_empty((4, 5))
    assert e.value.status == 3  # TG_E_NOMEM: no page-locked memory without a device
