"""Host-side logic of the batch paths, without a GPU: the read sizes a caller
derives from its call lists, and cy_render_traces's argument checks."""
import ctypes

import numpy as np
import pytest

from canvas_ity_gb300 import native, scenes
from canvas_ity_gb300 import trace as T
import golden_util as G


def _no_gpu():
    try:
        import torch
        return not torch.cuda.is_available()
    except ImportError:
        return True


@pytest.mark.parametrize("entry", G.manifest()[::5], ids=[e["name"] for e in G.manifest()[::5]])
def test_read_bytes_match_recorded_reads(entry):
    """trace.read_bytes (what a replay reads back) equals the bytes the
    reference recorded for the same get_image_data calls."""
    tb = G.load_fixture(entry)
    want = sum(img.nbytes for _, _, img in T.parse(tb).expected_images())
    assert T.read_bytes(tb) == want


def test_read_bytes_of_workload_canvas():
    tb = scenes.c3_canvas(11)
    w, h = T.canvas_size(tb)
    assert T.read_bytes(tb) == w * h * 4   # one full-canvas read at the end


def _render_traces_fn():
    lib = native.load()
    fn = lib.cy_render_traces
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_longlong,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return fn


def test_render_traces_rejects_bad_arguments():
    fn = _render_traces_fn()
    assert fn(None, None, 0, 0, 0, None, None, None) == 0          # nothing to do
    assert fn(None, None, -1, 0, 0, None, None, None) == -1        # negative count
    offs = np.zeros(2, np.uint64)
    assert fn(None, None, 1, 0, 0, None, offs.ctypes.data, None) == -1   # no call lists


@pytest.mark.skipif(not _no_gpu(), reason="a GPU is present")
def test_render_traces_without_device_reports_enodev():
    tb = scenes.small_scene("c0_small", 0)
    with pytest.raises(RuntimeError, match="status -4"):
        native.render_traces([tb])
