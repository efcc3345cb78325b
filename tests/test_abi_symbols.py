"""The C-ABI library builds for sm_103a, loads, and exports every entry point
include/xpsi_gb300.h declares.  No compute call is made (CPU-only check)."""
import ctypes
import os
import re
import shutil

import pytest

from conftest import ROOT


def declared_functions():
    txt = open(os.path.join(ROOT, "include", "xpsi_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(xgpu_[a-z0-9_]+)\s*\(", txt)))


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="nvcc not available")
def test_library_exports_header_symbols():
    from xpsi_gb300 import _native
    path = _native.build()
    lib = ctypes.CDLL(path)
    names = declared_functions()
    assert len(names) >= 13
    for n in names:
        getattr(lib, n)
    assert set(names) == set(_native.EXPORTED)
    assert lib.xgpu_abi_version() == _native.ABI_VERSION == 4
