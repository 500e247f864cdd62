"""The C ABI: the library loads, exports every declared entry point, and the
Python mirror of the header agrees with it.  No CUDA compute is called here."""

import ctypes as C
import os
import re

import numpy as np
import pytest

from braincell_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "braincell_gb300.h")
INCLUDE = os.path.join(ROOT, "include")


def _header_text():
    return open(HEADER).read()


def declared_functions():
    """Entry points declared in every header under include/ (the stable ABI and the
    tuning-diagnostics header)."""
    names = set()
    for fn in sorted(os.listdir(INCLUDE)):
        if fn.endswith(".h"):
            txt = open(os.path.join(INCLUDE, fn)).read()
            names |= set(re.findall(r"^\s*(?:bc_status|const char\*|int32_t|int64_t|void)\s+(bc_[a-z0-9_]+)\s*\(", txt, re.M))
    return sorted(names)


def test_debug_entry_points_stay_out_of_the_stable_header():
    assert "bc_debug_phase_cycles" not in _header_text()
    assert "bc_debug_phase_cycles" in declared_functions()


def test_every_declared_symbol_is_exported(native_lib):
    names = declared_functions()
    assert len(names) >= 18
    for n in names:
        assert hasattr(native_lib, n), f"{n} declared in the header but not exported"
        assert n in _abi.SIGNATURES, f"{n} has no ctypes signature"


def test_header_constants_match_python_mirror():
    txt = _header_text()
    found = 0
    for name, val in re.findall(r"#define\s+(BC_[A-Z0-9_]+)\s+(.+?)(?:\s*/\*|$)", txt, re.M):
        val = val.strip()
        m = re.fullmatch(r"\(1u << (\d+)\)", val)
        if m:
            v = 1 << int(m.group(1))
        elif re.fullmatch(r"0x[0-9a-fA-F]+u?", val):
            v = int(val.rstrip("u"), 16)
        elif re.fullmatch(r"-?\d+", val):
            v = int(val)
        else:
            continue
        if hasattr(_abi, name):
            assert getattr(_abi, name) == v, name
            found += 1
    assert found > 60


def test_struct_sizes(native_lib):
    # option / info structs have fixed 64-bit-friendly layouts
    assert C.sizeof(_abi.PlanOptions) == 4 * 16
    assert C.sizeof(_abi.PlanInfo) == 8 * 6 + 4 * 4 + 8 * 4 + 4 * 8


def test_version_and_defaults(native_lib):
    assert native_lib.bc_version() == _abi.BC_ABI_VERSION
    o = _abi.PlanOptions()
    native_lib.bc_default_options(C.byref(o))
    assert o.precision == _abi.BC_PREC_F32 and o.record_every == 1 and o.lane_nodes > 0


def test_invalid_spec_is_rejected_on_host(native_lib):
    s = _abi.BatchSpec()  # n_cells = 0
    h = C.c_void_p()
    st = native_lib.bc_plan_create(C.byref(s), None, C.byref(h))
    assert st == _abi.BC_ERR_INVALID
    assert b"n_cells" in native_lib.bc_last_error()


def test_null_plan_arguments(native_lib):
    assert native_lib.bc_plan_destroy(None) == _abi.BC_ERR_INVALID
    assert native_lib.bc_run(None, 1, 0.025, None) == _abi.BC_ERR_INVALID


def test_loader_refuses_another_abi_version(native_lib, monkeypatch):
    # a library whose records are laid out for another version must not be used
    monkeypatch.setattr(_abi, "_lib", None)
    monkeypatch.setattr(_abi, "BC_ABI_VERSION", _abi.BC_ABI_VERSION + 1)
    with pytest.raises(ImportError, match="ABI version"):
        _abi.lib()
    monkeypatch.undo()
    assert _abi.lib() is not None and _abi.lib().bc_version() == _abi.BC_ABI_VERSION
