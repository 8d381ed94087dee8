"""The C-ABI library loads and exports every symbol include/*.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import glob
import os
import re

from whatprot_gb300 import capi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(?:wp_status|void|void\*|const char\*|long long)\s+(wp_\w+)\s*\(", src):
            names.add(m.group(1))
    return names


def test_header_symbols_exported():
    lib = capi.load_library()
    names = declared_symbols()
    assert len(names) >= 10
    for n in sorted(names):
        assert hasattr(lib, n), n
    assert set(capi.EXPORTS) <= names


def test_no_cpu_fallback_when_missing(tmp_path):
    import pytest
    with pytest.raises(ImportError):
        capi.load_library(str(tmp_path / "missing.so"))
