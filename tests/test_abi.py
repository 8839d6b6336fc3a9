"""C-ABI checks that need no GPU: the library loads, exports every entry point the header
declares, and the ctypes descriptor layout matches the C struct."""
import ctypes
import os
import re

from opensbli_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "osb_gb300.h")).read()
    return sorted(set(re.findall(r"^int (osb_\w+)\(", txt, re.M)))


def test_header_and_binding_agree():
    assert header_functions() == sorted(abi.EXPORTED)


def test_library_exports_every_symbol(built_lib):
    lib = abi.load_library()
    for name in header_functions():
        assert hasattr(lib, name), name


def test_descriptor_layout(built_lib):
    lib = abi.load_library()
    out = (ctypes.c_longlong * 13)()
    assert lib.osb_desc_layout(out, 13) == 0
    assert list(out) == abi.layout_signature()


def test_version_and_errors(built_lib):
    lib = abi.load_library()
    assert lib.osb_version() == 100
    assert lib.osb_desc_layout(None, 0) == abi.OSB_EINVAL
    assert "13 slots" in abi.last_error(lib)
