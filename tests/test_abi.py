"""The C-ABI library loads and exports every entry point include/*.h declares (no GPU use)."""
import re
from pathlib import Path

import blochlib_gb300 as bl

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(bl_[a-z0-9_]+)\s*\(", txt):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = bl.load()
    names = declared_symbols()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binds_every_declared_symbol():
    assert set(declared_symbols()) <= set(bl._SIGS)


def test_version_and_error_string():
    lib = bl.load()
    assert b"sm_103a" in lib.bl_version()
    assert lib.bl_last_error() is not None
