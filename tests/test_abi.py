"""The C-ABI library loads and exports every function include/dmd.h
declares (CPU only: no compute call)."""
import ctypes as C
import os
import re

from dmdgb import abi

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "dmd.h")


def declared():
    text = open(HDR).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dmd_[a-z_0-9]+)\s*\(", text)))


def test_header_lists_entry_points():
    names = declared()
    assert "dmd_create" in names and "dmd_run" in names and "dmd_batch_run" in names
    assert set(abi.ENGINE_SYMBOLS) == set(names)


def test_library_exports_all(built):
    lib = abi.load_engine()
    for n in declared():
        assert hasattr(lib, n), n
    assert lib.dmd_version().decode().startswith("dmd-gb300")


def test_errors_are_status_codes(built):
    """Bad input returns a negative status and a message; nothing exits."""
    lib = abi.load_engine()
    h = C.c_void_p()
    cfg = abi.RunCfg(0.2, 1, 1, 1, 2000, 2, 1.2, 5e-5, 150.0, 0, 0)
    t = abi.Tables()
    s = abi.System()  # empty system
    rc = lib.dmd_create(C.byref(cfg), C.byref(t), C.byref(s), C.byref(h))
    assert rc == -1
    assert b"empty" in lib.dmd_last_error(h)
    lib.dmd_destroy(h)
