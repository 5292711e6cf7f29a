"""The C-ABI library loads and exports every function include/*.h declares
(no compute calls: this runs without a GPU)."""
import ctypes as C
import os
import re

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def declared():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(cl2pt_\w+|[a-z]\w*)\s*\(", src, re.M):
            name = m.group(1)
            if name in ("if", "for", "while", "sizeof", "return"):
                continue
            names.add(name)
    return sorted(names)


def test_library_exports_every_declared_symbol():
    from cl2pt import build
    path = build.build()
    lib = C.CDLL(path)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_declarations_found():
    names = declared()
    assert "cl2pt_plan_create" in names and "cl2pt_eval_real" in names
