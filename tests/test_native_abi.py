"""The C-ABI library builds, loads, and exports every function include/pamo_gb300.h declares (no GPU calls)."""

import os
import re
import subprocess

from pamo_gb300 import _native

HEADER = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include", "pamo_gb300.h")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pamo_[a-z0-9_]+)\s*\(", src)))


def test_header_symbols_exported(native_lib):
    names = declared()
    assert len(names) >= 10
    out = subprocess.run(["nm", "-D", "--defined-only", _native.lib_path()], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (pamo_[a-z0-9_]+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(native_lib, n)
    assert set(names) == set(_native.SIGNATURES), "ctypes signatures out of sync with the header"


def test_status_strings(native_lib):
    assert native_lib.pamo_status_string(0) == b"ok"
    assert native_lib.pamo_status_string(3) == b"capacity exceeded"
