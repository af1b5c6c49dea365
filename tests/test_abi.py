"""The C-ABI library builds, loads without a GPU, and exports every entry point
declared in include/*.h; host-side argument checking works without a device."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            text = open(os.path.join(ROOT, "include", f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(pq_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from polyquant_gb300 import build, _lib

    build.build()
    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 14
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(lib):
    from polyquant_gb300 import _lib

    assert set(_lib.EXPORTS) == set(declared_functions())


def test_version_and_null_arguments(lib):
    from polyquant_gb300 import _lib

    assert b"sm_103a" in lib.pq_version()
    h = ctypes.c_void_p()
    assert lib.pq_ci_create(None, None, ctypes.byref(h)) == _lib.PQ_ERR_ARG
    assert b"NULL" in lib.pq_last_error()
    assert lib.pq_ci_num_dets(None, None) == _lib.PQ_ERR_ARG
    assert lib.pq_ao2mo(None, 0, 1, 1, None, 1, 1, None, 1, 1, 0, None, None) == _lib.PQ_ERR_ARG


def test_desc_layout_matches_oracle():
    """pq_ci_desc and the oracle's descriptor share one field layout."""
    import oracle as O
    from polyquant_gb300 import _lib

    assert ctypes.sizeof(_lib.PQDesc) == ctypes.sizeof(O.OrcDesc)
    for (n1, t1), (n2, t2) in zip(_lib.PQDesc._fields_, O.OrcDesc._fields_):
        assert n1 == n2 and getattr(_lib.PQDesc, n1).offset == getattr(O.OrcDesc, n2).offset
