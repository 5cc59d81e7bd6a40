"""CPU checks of the C ABI library: it builds for sm_103a, loads, and exports
every entry point that include/spiralpir.h declares (no compute calls)."""
import ctypes
import os
import subprocess

from spiralpir import build, lib


def test_library_builds_and_loads():
    path = build.build()
    assert os.path.exists(path)
    ctypes.CDLL(path)


def test_exports_every_declared_symbol():
    path = build.build()
    declared = lib.header_symbols()
    assert declared, "no declarations parsed"
    h = ctypes.CDLL(path)
    for name in declared:
        assert hasattr(h, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert set(declared) <= exported
    assert set(lib.exported_symbols()) == set(declared)
