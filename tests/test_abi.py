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


def test_match_record_layout_matches_header():
    """gpu.MATCH_DTYPE mirrors blg_match (include/bitlev_gb300.h): int64
    query, int64 choice, int32 dist, int32 reserved, 24 bytes."""
    from editdist_bench_gb300 import gpu
    text = open(os.path.join(ROOT, "include", "bitlev_gb300.h")).read()
    body = re.search(r"typedef struct \{([^}]*)\} blg_match;", text).group(1)
    fields = re.findall(r"(int64_t|int32_t)\s+(\w+);", body)
    assert fields == [("int64_t", "query"), ("int64_t", "choice"), ("int32_t", "dist"), ("int32_t", "reserved")]

    class M(ctypes.Structure):
        _fields_ = [("query", ctypes.c_int64), ("choice", ctypes.c_int64), ("dist", ctypes.c_int32),
                    ("reserved", ctypes.c_int32)]
    assert gpu.MATCH_DTYPE.itemsize == ctypes.sizeof(M) == 24
    assert [gpu.MATCH_DTYPE.fields[n][1] for n in ("query", "choice", "dist", "reserved")] == \
        [M.query.offset, M.choice.offset, M.dist.offset, M.reserved.offset]


def test_matches_reject_exact_runs_before_any_device_call():
    """A matches-only search needs max_dist (the exact result is the dense
    cdist); the check runs in Python, so it raises without a GPU too."""
    from editdist_bench_gb300 import gpu
    with pytest.raises(ValueError):
        gpu.cdist_matches(["ACGT"], ["ACGA"], None)
    with pytest.raises(ValueError):
        gpu.cdist_matches(["ACGT"], ["ACGA"], -1)
