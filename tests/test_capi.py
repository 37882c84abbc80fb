"""The C-ABI library builds for sm_103a, loads, and exports every entry point
include/folgb.h declares (no compute calls: no GPU needed)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "folgb.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(folgb_\w+)\s*\(", src)))


def test_header_declares_the_boundary():
    syms = declared_symbols()
    for name in ("folgb_plan_create", "folgb_loss_adjoint", "folgb_assemble", "folgb_pcg", "folgb_adam_step",
                 "folgb_batch_loss_adjoint"):
        assert name in syms


def test_library_exports_every_declared_symbol():
    from folax_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_header():
    from folax_gb300 import _capi
    assert set(declared_symbols()) == set(_capi.PROTOTYPES)
