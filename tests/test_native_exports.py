"""The C-ABI library builds for sm_103a, loads without a GPU, and exports every declared symbol."""

import ctypes
import os
import re

from pyseqm_gb300 import build, native

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "pyseqm_gb300.h")


def _declared():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(seqm_\w+)\s*\(", src, re.M)))


def test_header_matches_binding_list():
    assert _declared() == sorted(native.EXPORTS)


def test_library_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    for name in _declared():
        assert hasattr(lib, name), name
    native.load(path)
    assert b"sm_103a" in native.load().seqm_version()
