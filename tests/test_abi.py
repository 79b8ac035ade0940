"""The C ABI library loads without a GPU and exports every function that
include/acg.h and include/acg_io.h declare; the ctypes table covers them all."""
import re

from application_classification_gb300 import _lib, build

DECL = re.compile(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(acg_[a-z0-9_]+)\s*\(", re.M)


def declared():
    names = set()
    for h in sorted((build.ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(DECL.findall(text))
    return names


def test_every_declared_symbol_is_exported():
    names = declared()
    assert len(names) >= 25, names
    L = _lib.lib()
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing


def test_ctypes_table_covers_the_headers():
    assert declared() == set(_lib.SIGNATURES)


def test_version_and_status_strings():
    L = _lib.lib()
    assert L.acg_version().decode().startswith("acg ")
    assert L.acg_status_string(0).decode()
    assert L.acg_status_string(999).decode()  # unknown codes still give a string
