"""The C ABI library loads and exports every entry point include/*.h declares (CPU only:
no kernel is launched here)."""
import ctypes
import glob
import os
import re

import pytest

from fdf_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(fdf_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "fdf_AdvanceStep" in names and "fdf_SetGrid" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(build.build())
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_python_binding_covers_the_header():
    assert set(declared_functions()) == set(_lib.exported_symbols())


def test_python_constants_match_the_header():
    """The Python mirror's form, route and locator constants are the header's #defines."""
    from fdf_gb300 import context as C
    defines = {}
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        for name, val in re.findall(r"^#define\s+FDF_(\w+)\s+(-?\d+)\s*$", open(h).read(), flags=re.M):
            defines[name] = int(val)
    pairs = {"FORM_PLAIN_FP64": C.FORM_PLAIN_FP64, "FORM_FP32": C.FORM_FP32, "FORM_LEARNED_FP32": C.FORM_LEARNED_FP32,
             "TRANSFER_STAGED": C.TRANSFER_STAGED, "TRANSFER_IN_PLACE": C.TRANSFER_IN_PLACE,
             "TRANSFER_AUTO": C.TRANSFER_AUTO, "LOCATOR_BF16": C.LOCATOR_BF16, "LOCATOR_F16": C.LOCATOR_F16,
             "LOCATOR_NPARAM": C.LOCATOR_NPARAM}
    for name, value in pairs.items():
        assert defines[name] == value, name


def test_context_create_fails_loudly_without_gpu():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    lib = _lib.load()
    h = ctypes.c_void_p()
    rc = lib.fdf_ContextCreate(ctypes.byref(h), 0)
    assert rc == 97 and not h.value   # PETSC_ERR_GPU, no context


def test_null_arguments_rejected():
    lib = _lib.load()
    assert lib.fdf_ContextCreate(None, 0) == 85        # PETSC_ERR_ARG_NULL
    assert lib.fdf_SetTimeStep(None, 1.0) == 85
    assert lib.fdf_AdvanceStep(None, None) == 85
