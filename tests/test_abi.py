"""The C-ABI library builds, loads without a GPU, and exports every symbol
that include/*.h declares.  No compute call is made here."""
import ctypes
import glob
import os
import re

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(qcmg_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    from pyqcm_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.qcmg_version


def test_python_binding_covers_header():
    from pyqcm_gb300 import _lib
    assert declared_symbols() == set(_lib.exported_symbols())


def test_errors_are_reported_without_gpu():
    from pyqcm_gb300 import _lib
    lib = _lib.lib()
    # argument errors are detected before any device work
    d = ctypes.c_size_t()
    assert lib.qcmg_halfbasis(40, 3, None, 0, ctypes.byref(d)) == -1
    assert "L must be" in _lib.last_error()
    lib.qcmg_version.restype = ctypes.c_char_p
    assert lib.qcmg_version().startswith(b"qcmg")
