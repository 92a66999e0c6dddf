"""CPU: the C-ABI library loads and exports every symbol include/*.h declares."""
import ctypes
import os
import re

from litert_gb300 import lrt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if not name.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", name)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(lrt_[a-z0-9_]+)\s*\(", text):
            syms.add(m.group(1))
    return syms


def test_library_exports_declared_symbols():
    syms = declared_symbols()
    assert len(syms) > 20
    L = ctypes.CDLL(lrt.LIB_PATH)
    missing = [s for s in sorted(syms) if not hasattr(L, s)]
    assert not missing, missing


def test_status_strings_and_camera_helpers():
    L = lrt.lib()
    assert L.lrt_status_string(0) == b"ok"
    m = lrt.look_at((0, 0, 3), (0, 0, 0), (0, 1, 0))
    inv = lrt.inverse4x4(m)
    import numpy as np
    assert np.allclose(m @ inv, np.eye(4), atol=1e-6)
    # camera at (0,0,3): world origin maps to view-space (0,0,-3)
    assert np.allclose(m @ np.array([0, 0, 0, 1], np.float32), [0, 0, -3, 1], atol=1e-6)


def test_create_without_gpu_fails_cleanly():
    """lrt_create reports an error code instead of crashing when no device is usable."""
    import torch
    if torch.cuda.is_available():
        return
    ctx = ctypes.c_void_p()
    st = lrt.lib().lrt_create(ctypes.byref(ctx), 0)
    assert st != 0 and not ctx.value
