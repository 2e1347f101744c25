"""The C ABI: the library builds for sm_103a, loads without a GPU, and exports
every function ``include/zandgpu.h`` declares (no compute calls here)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "zandgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(zg_[A-Za-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def libpath():
    from zandpack_gb300 import build
    if not os.path.exists(build.LIB):
        build.build()
    return build.LIB


def test_header_symbols_exported(libpath):
    L = ctypes.CDLL(libpath)
    names = _declared()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_binding_covers_header(libpath):
    from zandpack_gb300 import _lib
    assert sorted(_lib.exported_symbols()) == _declared()
    assert _lib.lib().zg_version() >= 100


def test_invalid_arguments_fail_loudly(libpath):
    """Argument checks run on the host before any device work."""
    from zandpack_gb300 import _lib
    L = _lib.lib()
    st = L.zg_traj_create(0, None, 0, None)
    assert st == _lib.ZG_EINVAL
    assert b"null" in L.zg_last_error()
    with pytest.raises(AssertionError):
        _lib.check(st)
