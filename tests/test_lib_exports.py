"""The C-ABI library builds for sm_103a, loads, and exports every declared symbol (no GPU calls)."""
import ctypes
import os
import re

import pytest

from fermicg_gb300 import build, gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(fcg_[a-z0-9_]+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol():
    path = build.build()
    L = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 10
    for s in sorted(syms):
        assert hasattr(L, s), s
    assert syms <= set(gpu.SIGNATURES), syms - set(gpu.SIGNATURES)


def test_binding_loads_and_reports_version():
    L = gpu.load_library()
    assert L.fcg_version() >= 1
