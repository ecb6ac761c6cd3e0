"""The C-ABI library builds for sm_103a, loads without a GPU, and exports every
function include/*.h declares.  No compute call is made here."""
import glob
import os
import re

import ctypes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ \*]*?\b(ddla_[a-z0-9_]+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


def test_library_builds_and_exports_header(ddla):
    L = ctypes.CDLL(ddla._lib.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing


def test_python_binding_covers_header(ddla):
    assert declared_functions() <= set(ddla._lib.exported_names())


def test_version_string(ddla):
    assert ddla.lib().ddla_version().startswith(b"ddla_gb300")


def test_oracle_is_not_linked_into_product():
    prod = open(os.path.join(ROOT, "ddla_gb300", "_build", "libddla_gb300.so"), "rb").read()
    assert b"orc_dgemm" not in prod
    # no product source imports, loads or calls the oracle (comments may name
    # it; code may not use it)
    uses = re.compile(r"(from\s+oracle\b|import\s+oracle\b|libddla_oracle|\borc_[a-z]|oracle/|oracle\.)")
    for src in glob.glob(os.path.join(ROOT, "ddla_gb300", "**", "*.*"), recursive=True) + \
            glob.glob(os.path.join(ROOT, "include", "*.h")):
        if src.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
            code = "\n".join(ln.split("#")[0] if src.endswith(".py") else ln.split("//")[0]
                             for ln in open(src).read().splitlines())
            hit = uses.search(code)
            assert hit is None, f"{src} uses the oracle: {hit.group(0)!r}"

