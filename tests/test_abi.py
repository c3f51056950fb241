"""The C-ABI library builds, loads and exports every entry point declared in
include/*.h (no compute call: this runs without a GPU)."""
import ctypes as C
import re
from pathlib import Path

import pytest

from conftest import HAS_GPU, ROOT


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = h.read_text()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names |= set(re.findall(r"\b(ent_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("ent_create", "ent_destroy", "ent_densities", "ent_densities_device"):
        assert s in syms


def test_library_exports_all_declared():
    from entropical_gb300 import _build
    path = _build.build()
    lib = C.CDLL(str(path))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_signatures_cover_header():
    from entropical_gb300 import _native
    declared = set(declared_symbols())
    assert declared <= set(_native.SIGNATURES), declared - set(_native.SIGNATURES)


@pytest.mark.skipif(HAS_GPU, reason="checks the no-device path")
def test_no_device_is_an_error_not_a_fallback():
    from entropical_gb300 import Context, NativeError
    with pytest.raises(NativeError) as ei:
        Context()
    assert ei.value.status == 7  # ENT_ERR_NO_DEVICE
