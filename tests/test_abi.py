"""CPU: libflaregb loads and exports every symbol include/flaregb.h
declares; host-only argument checks return the documented status codes."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "flaregb.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fgb_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "fgb_predict" in syms and "fgb_nlist_build" in syms
    assert len(syms) >= 20


def test_library_exports_every_declared_symbol(flaregb_lib):
    for s in declared_symbols():
        assert hasattr(flaregb_lib, s), s


def test_python_binding_covers_header():
    from flare_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_b2_create_rejects_bad_settings(flaregb_lib):
    from flare_gb300 import _lib
    h = ctypes.c_void_p()
    rh = (ctypes.c_double * 2)(0.0, 5.0)
    rc = flaregb_lib.fgb_b2_create(ctypes.byref(h), 0, 0, rh, 2, None, 0, 1, 8,
                                   11, None)
    assert rc == _lib.FGB_EINVAL
    assert b"l_max" in flaregb_lib.fgb_last_error()
    rc = flaregb_lib.fgb_b2_create(ctypes.byref(h), 9, 0, rh, 2, None, 0, 1, 8,
                                   3, None)
    assert rc == _lib.FGB_EINVAL
    # weighted Chebyshev needs lambda = radial_hyps[2]
    rc = flaregb_lib.fgb_b2_create(ctypes.byref(h), 1, 0, rh, 2, None, 0, 1, 8,
                                   3, None)
    assert rc == _lib.FGB_EINVAL
    rc = flaregb_lib.fgb_b2_create(ctypes.byref(h), 5, 0, rh, 2, None, 0, 1, 8,
                                   3, None)
    assert rc == _lib.FGB_OK
    assert flaregb_lib.fgb_b2_destroy(h) == 0
    rc = flaregb_lib.fgb_b2_create(ctypes.byref(h), 0, 0, rh, 2, None, 0, 1, 8,
                                   3, None)
    assert rc == _lib.FGB_OK
    assert flaregb_lib.fgb_b2_destroy(h) == 0


def test_python_errors_map_to_reference_exceptions():
    import flare_gb300 as fg
    with pytest.raises(ValueError):
        fg.B2("legendre", "quadratic", [0, 5], [], [1, 8, 3])
    with pytest.raises(ValueError):
        fg.B2("chebyshev", "quadratic", [0, 5], [], [1, 8])
