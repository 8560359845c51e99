"""The C-ABI library loads on a machine without a GPU and exports every
entry point include/qslc.h declares (no compute calls here)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    txt = open(os.path.join(ROOT, "include", "qslc.h")).read()
    return sorted(set(re.findall(r"QSLC_API[^;(]*?\b(qslc_\w+)\s*\(", txt)))


def test_header_declares_the_api():
    names = declared()
    for must in ("qslc_create", "qslc_create_np", "qslc_gate1", "qslc_gate2", "qslc_prob",
                 "qslc_sample_all", "qslc_measure", "qslc_get_state", "qslc_set_state"):
        assert must in names


def test_library_exports_every_declared_symbol(qsl):
    lib = ctypes.CDLL(qsl.LIB_PATH)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", qsl.LIB_PATH], capture_output=True,
                         text=True).stdout
    exported = set(re.findall(r" T (qslc_\w+)", out))
    assert set(declared()) <= exported
    assert exported <= set(declared()), exported - set(declared())


def test_python_binding_covers_the_header(qsl):
    assert set(qsl.SIGNATURES) == set(declared())
    lib = qsl.lib()
    assert lib.qslc_version() == 100
    assert lib.qslc_last_error() == b""
