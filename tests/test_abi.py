"""The C-ABI library loads and exports every function include/*.h declares
(no compute calls: this runs without a GPU)."""
import ctypes as C
import os
import re

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def declared(only=None, skip=()):
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if not f.endswith(".h") or f in skip or (only and f != only):
            continue
        src = open(os.path.join(ROOT, "include", f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z]\w*)\s*\(", src, re.M):
            name = m.group(1)
            if name in ("if", "for", "while", "sizeof", "return"):
                continue
            names.add(name)
    return sorted(names)


def test_library_exports_every_declared_symbol():
    from cl2pt import build
    path = build.build()
    lib = C.CDLL(path)
    missing = [n for n in declared(skip=("cl2pt_legacy.h",)) if not hasattr(lib, n)]
    assert not missing, missing


def test_legacy_library_exports_the_reference_names():
    """libcl2pt_legacy.so exports every name cl2pt_legacy.h declares, among
    them the reference's cosmo2D.h / pt_cfastpt.h / cfastpt.h entry points."""
    from cl2pt import build
    build.build()
    lib = C.CDLL(build.LEGACY)
    names = declared(only="cl2pt_legacy.h")
    for ref in ("xi_pm_tomo", "w_gammat_tomo", "w_gg_tomo", "C_ss_tomo_limber", "C_cl_tomo",
                "get_FPT_bias", "get_FPT_IA", "J_abl", "J_abJ1J2Jk"):
        assert ref in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    for g in ("FPTbias", "FPTIA"):
        assert hasattr(lib, g)


def test_declarations_found():
    names = declared()
    assert "cl2pt_plan_create" in names and "cl2pt_eval_real" in names
