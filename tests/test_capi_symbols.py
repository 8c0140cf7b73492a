"""The C-ABI library loads and exports every entry point include/asg_gb300.h declares.

CPU-only: no compute call is made (there is no GPU here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "asg_gb300.h")
LIB = os.path.join(ROOT, "angularspectrum_heterogeneous_gb300", "libasgb300.so")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(asg_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared()
    for must in ["asg_plan_create", "asg_plan_destroy", "asg_set_step_operators",
                 "asg_add_screen", "asg_add_source", "asg_run", "asg_get_outputs",
                 "asg_apply_operator", "asg_flux_columns", "asg_last_error"]:
        assert must in names


def test_library_exports_all_declared_symbols():
    if not os.path.exists(LIB):
        import __graft_entry__ as g
        g.build()
    lib = ctypes.CDLL(LIB)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_matches_header():
    from angularspectrum_heterogeneous_gb300 import _lib
    assert sorted(_lib.EXPORTED) == sorted(n for n in declared()), "ctypes binding out of date"


def test_version_string_without_gpu():
    lib = ctypes.CDLL(LIB)
    lib.asg_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.asg_version()
