"""The C-ABI library loads without a GPU and exports every symbol that
include/igsolve.h declares; the ctypes table covers the same set.  No compute
call is made here."""
import os
import re
import subprocess

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "igsolve.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ig_\w+)\s*\(", src)))


def test_header_declares_the_abi():
    names = _declared()
    for must in ("ig_solve3d", "ig_solve3d_mg", "ig_solve3d_vmg",
                 "ig_solve_basis_vmg", "ig_sweep_dev", "ig_request_stop"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from ion_gym_gb300 import _lib
    L = _lib.lib()
    for name in _declared():
        assert hasattr(L, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH],
                         capture_output=True, text=True).stdout
    exported = set(re.findall(r"\sT\s(ig_\w+)", out))
    assert set(_declared()) <= exported


def test_ctypes_table_matches_header():
    from ion_gym_gb300 import _lib
    assert set(_lib.SIGNATURES) == set(_declared())


def test_loads_without_a_device():
    from ion_gym_gb300 import _lib
    L = _lib.lib()
    assert L.ig_abi_version() == 2
    assert L.ig_device_count() >= 0
    L.ig_request_stop()
    assert L.ig_stop_requested() == 1
    L.ig_clear_stop()
    assert L.ig_stop_requested() == 0
