"""The C ABI: library loads, exports what include/*.h declares, host-side paths."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(wr_[a-z_]+)\s*\(", text))
    return names


def test_exports_every_declared_symbol(wr):
    lib = wr.lib()
    declared = _declared()
    assert {"wr_create", "wr_run", "wr_prepare", "wr_advance", "wr_upload", "wr_download"} <= declared
    for name in declared:
        assert hasattr(lib, name), name
    # and nm agrees: they are real dynamic symbols
    out = subprocess.run(["nm", "-D", "--defined-only", wr.LIB_PATH], capture_output=True, text=True).stdout
    for name in declared:
        assert re.search(rf"\bT {name}\b", out), name


def test_struct_layouts(wr):
    assert wr.COLLAPSE_STATE.itemsize == 216
    assert wr.PACKED_FINAL_STATE.itemsize == 172


def test_initial_state_matches_reference(wr, oracle_libm):
    """wr_make_collapse_state is host code: bitwise the reference's
    make_collapse_state (reproducer.cpp:7533-7546) as restated by the oracle."""
    a = wr.make_collapse_state()
    b = oracle_libm.make_collapse_state()
    assert a.tobytes() == b.tobytes()
    assert a["T"] == 100.0 and a["completed_steps"] == 0 and a["density_driver"] == a["rho"]


def test_bad_arguments_fail_before_any_device_call(wr):
    h = ctypes.c_void_p()
    assert wr.lib().wr_create(0, 0, wr.MATH_PORTABLE, ctypes.byref(h)) == wr.BAD_INPUTS
    assert "num_cells" in wr.last_error()
    assert wr.lib().wr_create(8, 0, 7, ctypes.byref(h)) == wr.BAD_INPUTS
    assert wr.lib().wr_run(None, 1, None) == wr.BAD_INPUTS


def test_packed_record_round_trip(wr):
    """tests/integration/test_grid_timestep_reference.mojo:142-168 restated: cell 23
    of a grid-4 run packs to i, j, k = 3, 1, 1."""
    c = np.zeros(24, wr.COLLAPSE_STATE)
    s = c[23]
    s["completed_steps"] = 17
    s["time"] = 123.5
    s["density_driver"] = 4.25e-9
    s["rho"] = 9.5
    s["T"] = 88.0
    s["e"] = -3.25
    s["xn"] = np.arange(14) + 0.125
    p = wr.pack_final_states(c, 4)[23]
    raw = p.tobytes()
    assert len(raw) == 172
    d = np.frombuffer(raw, wr.PACKED_FINAL_STATE)[0]
    assert (d["cell"], d["i"], d["j"], d["k"], d["completed_steps"]) == (23, 3, 1, 1, 17)
    assert (d["time"], d["density_driver"], d["rho"], d["T"], d["e"]) == (123.5, 4.25e-9, 9.5, 88.0, -3.25)
    assert (d["xn"] == np.arange(14) + 0.125).all()
