"""The C-ABI library loads and exports every symbol include/*.h declares;
without a GPU the entry points report "no device" instead of crashing."""
import ctypes
import glob
import os
import re

import pytest

from editdist_bench_gb300 import _build, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        names.update(re.findall(r"\b(blg_[a-z0-9_]+)\s*\(", text))
    return names


@pytest.fixture(scope="module")
def lib():
    return ctypes.CDLL(_build.build())


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert {"blg_init", "blg_pairwise", "blg_cdist", "blg_pairs_run", "blg_search_run"} <= names
    for n in sorted(names):
        assert hasattr(lib, n), f"{n} declared in include/ but not exported"


def test_ctypes_signatures_cover_the_header():
    assert {s[0] for s in _lib.SIGNATURES} >= _declared()


def test_library_reports_no_device_without_gpu(lib):
    L = _lib.load()
    assert L.blg_version() >= 100
    n = L.blg_device_count()
    if n == 0:
        h = ctypes.c_void_p()
        assert L.blg_init(0, ctypes.byref(h)) == _lib.ERR_NODEVICE
        assert L.blg_pairs_run(None, None, -1, 0, None) == _lib.ERR_ARG
        assert L.blg_last_error(None) == b"no context"


def test_product_package_does_not_import_oracle():
    pkg = os.path.join(ROOT, "editdist_bench_gb300")
    for path in glob.glob(os.path.join(pkg, "**", "*.*"), recursive=True):
        if path.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
            text = open(path, encoding="utf-8").read()
            assert not re.search(r"^\s*(import|from)\s+oracle\b", text, flags=re.M), path
            assert "liborc" not in text and "myers_oracle" not in text, path
