"""The C-ABI library loads and exports every symbol include/llfem_gb300.h
declares; host-only calls work without a GPU."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "llfem_gb300.h")).read()
    return sorted(set(re.findall(r"\b(llf_[a-z0-9_]+)\s*\(", src)))


def test_exports_every_declared_symbol(llf):
    lib = ctypes.CDLL(llf._lib.LIBPATH)
    names = _declared()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_rule_host_only(llf):
    assert llf._lib.lib().llf_version().decode().count(".") == 2
    r = llf._lib.builtin_rule(5, 2)
    assert r["nip"] == 27 and r["npe"] == 27


def test_unsupported_rule_is_an_error(llf):
    with pytest.raises(llf.LLFError):
        llf._lib.builtin_rule(5, 7)


def test_null_arguments_rejected(llf):
    L = llf._lib.lib()
    assert L.llf_ctx_create(0, None) == -1
    assert L.llf_pcg(None, None, None, None, None, 0, 1e-8, 1, None, None) == -1
