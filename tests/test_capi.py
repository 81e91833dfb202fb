"""The C ABI: the library loads, exports every declared symbol, and turns
bad arguments into status codes without touching the GPU."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    text = (ROOT / "include/lvrgb.h").read_text()
    return sorted(set(re.findall(r"\b(lvrgb_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_binding_list():
    from lvr2_gb300._lib import EXPORTS
    assert sorted(EXPORTS) == declared_functions()


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name


def test_version_and_error_strings(lib):
    assert b"sm_103a" in lib.lvrgb_version()
    assert isinstance(lib.lvrgb_last_error(), bytes)


def test_invalid_arguments_return_status(lib):
    from lvr2_gb300._lib import SurfaceConfig
    cfg = SurfaceConfig()
    lib.lvrgb_surface_config_default(ctypes.byref(cfg))
    assert (cfg.kn, cfg.ki, cfg.kd, cfg.nem) == (10, 10, 5, 0)
    h = ctypes.c_void_p()
    pts = np.zeros((4, 3), np.float32)
    # negative size
    st = lib.lvrgb_surface_create(ctypes.byref(cfg), pts.ctypes.data_as(ctypes.c_void_p), -1, 0, None,
                                  ctypes.byref(h))
    assert st == 1 and h.value is None
    # plane-fit methods are 0..4
    cfg.nem = 5
    st = lib.lvrgb_surface_create(ctypes.byref(cfg), pts.ctypes.data_as(ctypes.c_void_p), 4, 0, None,
                                  ctypes.byref(h))
    assert st == 1 and b"nem" in lib.lvrgb_last_error()
    cfg.nem = 3
    cfg.kn = 0
    st = lib.lvrgb_surface_create(ctypes.byref(cfg), pts.ctypes.data_as(ctypes.c_void_p), 4, 0, None,
                                  ctypes.byref(h))
    assert st == 1
    # NULL handle
    assert lib.lvrgb_calculate_normals(None, None) == 1
    assert lib.lvrgb_surface_destroy(None) == 0


def test_python_mirror_raises_on_status(lib):
    import lvr2_gb300
    with pytest.raises(lvr2_gb300.LvrgbError) as e:
        lvr2_gb300.Surface(np.zeros((4, 3), np.float32), nem=7)
    assert e.value.status == 1
