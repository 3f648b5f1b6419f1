"""The C-ABI library builds, loads without a GPU and exports every declared symbol."""
import ctypes
import os
import re

import pytest

from canvas_ity_gb300 import build, native

INCLUDE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "include")


def declared_functions():
    names = set()
    for h in ("cy_gpu.h", "canvas_ity_c.h", "cy_batch.h", "cy_serve.h"):
        path = os.path.join(INCLUDE, h)
        if not os.path.exists(path):
            continue
        text = open(path).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(cy_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_builds_and_loads():
    path = build.build()
    assert os.path.exists(path)
    lib = ctypes.CDLL(path)
    assert lib is not None


@pytest.mark.parametrize("name", declared_functions())
def test_symbol_exported(name):
    lib = ctypes.CDLL(build.build())
    assert hasattr(lib, name), f"{name} declared in include/ but not exported"


def test_no_device_is_reported_not_faked():
    """Without a GPU a canvas reports ENODEV instead of rendering elsewhere."""
    lib = native.load()
    lib.cy_canvas_new.restype = ctypes.c_void_p
    lib.cy_canvas_status.argtypes = [ctypes.c_void_p]
    lib.cy_canvas_delete.argtypes = [ctypes.c_void_p]
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    c = lib.cy_canvas_new(16, 16)
    assert c
    assert lib.cy_canvas_status(c) == -4
    lib.cy_canvas_delete(c)
