"""C-ABI checks that need no GPU: the library loads, exports every entry
point include/rg_api.h declares, and refuses to run without a device."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "rg_api.h")


def declared():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(rg_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def libpath():
    from openradioss_gb300 import build
    return build.build()


def test_every_declared_symbol_is_exported(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (rg_[a-z0-9_]+)\b", out))
    missing = [s for s in declared() if s not in exported]
    assert not missing, missing
    assert len(declared()) >= 25


def test_ctypes_signatures_cover_header(libpath):
    from openradioss_gb300 import _lib
    names = {n for n, _, _ in _lib.SIGNATURES}
    assert set(declared()) <= names | {"rg_skyline_get"} and set(declared()) == names


def test_no_device_fails_loudly(libpath):
    import ctypes as C
    from openradioss_gb300 import _lib
    L = _lib.lib(libpath)
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert L.rg_ctx_create(0, C.byref(h)) < 0
    assert not h.value


def test_engine_refuses_without_library(tmp_path):
    from openradioss_gb300 import _lib
    with pytest.raises(RuntimeError):
        _lib.lib(str(tmp_path / "missing.so"))


def test_fortran_module_binds_every_entry_point():
    """include/rg_api_mod.F90 (the ISO_C_BINDING module a Fortran engine
    uses) binds every function the C header declares, by its C name."""
    src = open(os.path.join(ROOT, "include", "rg_api_mod.F90")).read()
    bound = set(re.findall(r"bind\(c,\s*name='(rg_[a-z0-9_]+)'\)", src))
    missing = [s for s in declared() if s not in bound]
    assert not missing, missing
    assert bound <= set(declared()), sorted(bound - set(declared()))
