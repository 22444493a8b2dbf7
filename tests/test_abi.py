"""The C-ABI library builds, loads, and exports every entry point of include/eb_gb300.h.
No compute call is made here (these run without a GPU)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "eb_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*?\**\s*\b([a-z_][a-z0-9_]*)\s*\(",
                       src, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "for", "while", "return")))


def test_header_parses():
    names = header_functions()
    assert "eb_stokes_matvec" in names and "matvec_" in names and len(names) > 20


def test_library_exports_every_declared_symbol(eblib):
    missing = [n for n in header_functions() if not hasattr(eblib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from electricbubbles_gb300 import _lib
    assert set(header_functions()) == set(_lib.SIGNATURES)


def test_status_strings(eblib):
    assert eblib.eb_status_string(0) == b"ok"
    assert eblib.eb_version() == 6


def test_context_without_device_fails_loudly(eblib):
    import ctypes
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from electricbubbles_gb300 import EbError
    from electricbubbles_gb300.api import Context
    with pytest.raises(EbError) as e:
        Context()
    assert e.value.status == 8  # EB_ERR_NODEVICE


def test_oracle_is_not_imported_by_the_product():
    """The product package never references the oracle."""
    pkg = os.path.join(ROOT, "electricbubbles_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h")):
                txt = open(os.path.join(dirpath, f)).read()
                assert "eb_oracle" not in txt and "import oracle" not in txt, f
