"""The C-ABI library builds, loads, and exports every symbol include/*.h declares
(no compute without a GPU)."""
import glob
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"\b(ctw_[a-z0-9_]+)\s*\(", txt):
            syms.add(m.group(1))
    return syms


def test_library_exports_declared_symbols():
    from ctwin_gb300 import build
    lib = build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (ctw_[a-z0-9_]+)", out))
    declared = declared_symbols()
    assert declared, "no declarations found"
    missing = declared - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"


def test_library_loads_and_reports():
    from ctwin_gb300._native import lib
    L = lib()
    assert L.ctw_version().startswith(b"ctwin_gb300")
    assert L.ctw_device_count() >= 0


def test_create_fails_cleanly_without_gpu_or_bad_args():
    import ctypes
    from ctwin_gb300._native import lib
    L = lib()
    h = ctypes.c_void_p()
    assert L.ctw_prp_create(5, 1, ctypes.byref(h)) == -1        # degree out of range
    assert L.ctw_prp_create(11, 0, ctypes.byref(h)) == -1       # no lanes
    if L.ctw_device_count() == 0:
        assert L.ctw_prp_create(11, 1, ctypes.byref(h)) == -2   # CUDA error, not a crash
        assert b"no CUDA device" in L.ctw_last_error()


def test_argument_errors_are_reported_before_the_device_is_asked():
    """Invalid shapes give CTW_E_ARG (-1) with or without a GPU; valid ones
    without a GPU give CTW_E_CUDA (-2).  Nothing crashes, no handle is returned."""
    import ctypes
    from ctwin_gb300._native import lib
    L = lib()
    h = ctypes.c_void_p()
    assert L.ctw_prp_create_split(16, 1, 9, ctypes.byref(h)) == -1     # 2^16 on 512 CTAs: no kernel
    assert L.ctw_prp_create_split(18, 1, 2, ctypes.byref(h)) == -1     # 2^18 on 4 CTAs of 65536: no kernel
    assert L.ctw_prp_create_split(8, 1, 3, ctypes.byref(h)) == -1      # runs of 32 coefficients: none
    assert L.ctw_pool_create(12, 4, 9, 0, 2, 0, ctypes.byref(h)) == -1
    assert L.ctw_pool_create(12, 0, -1, 0, 2, 0, ctypes.byref(h)) == -1
    assert not h.value
    if L.ctw_device_count() == 0:
        assert L.ctw_prp_create_split(16, 1, 5, ctypes.byref(h)) == -2  # the 32-CTA grid exists
        assert L.ctw_pool_create(12, 4, -1, 0, 2, 0, ctypes.byref(h)) == -2
        assert not h.value
