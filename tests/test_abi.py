"""CPU checks of the drop-in boundary: the library loads and exports every
entry point include/va.h declares (no compute calls without a GPU)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for f in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            names += re.findall(r"^VA_API[^(]*?\b(va_\w+)\s*\(", src, flags=re.M)
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "va_forward" in names and "va_backward" in names and "va_gradient" in names
    assert len(names) == len(set(names))


def test_library_exports_every_declared_symbol(valib):
    lib = ctypes.CDLL(valib.LIB_PATH)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_lists_every_export(valib):
    from vectorizedadjoint_gb300 import _lib
    assert sorted(_lib.EXPORTS) == sorted(declared_symbols())


def test_default_options_and_status_strings(valib):
    L = valib.load()
    from vectorizedadjoint_gb300 import _lib
    o = _lib.VaOptions()
    assert L.va_default_options(ctypes.byref(o)) == 0
    assert o.max_rejects == 500 and o.tableau == 0 and o.precision == 0
    assert o.atol == 1e-6 and o.rtol == 1e-6 and o.dt0 == 1e-3
    assert L.va_status_string(4) == b"VA_CKPT_BUDGET"
    assert L.va_default_options(None) == 5


def test_create_rejects_bad_problems(valib):
    """Argument validation happens before any device call."""
    L = valib.load()
    from vectorizedadjoint_gb300 import _lib
    h = ctypes.c_void_p()
    o = _lib.VaOptions()
    L.va_default_options(ctypes.byref(o))
    bad = [_lib.VaProblem(0, 3, 1, 4, 1),   # VdP with n=3
           _lib.VaProblem(0, 2, 1, 0, 1),   # empty batch
           _lib.VaProblem(2, 2, 1, 4, 1),   # DHO with npar=1
           _lib.VaProblem(99, 2, 1, 4, 1)]  # unknown model
    for p in bad:
        assert L.va_create(ctypes.byref(p), ctypes.byref(o), ctypes.byref(h)) == 5
    o.tableau = 7
    p = _lib.VaProblem(0, 2, 1, 4, 1)
    assert L.va_create(ctypes.byref(p), ctypes.byref(o), ctypes.byref(h)) == 5
