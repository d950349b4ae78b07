"""The C-ABI library: it builds, loads and exports every symbol include/tracefem.h declares."""
import os
import re

import pytest

import drops_gb300 as tf

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "tracefem.h")).read()
    return sorted(set(re.findall(r"\b(tf_[a-z0-9_]+)\s*\(", text)))


def test_header_matches_python_export_list():
    assert declared_symbols() == sorted(tf.EXPORTS)


def test_library_loads_and_exports_all_symbols():
    from drops_gb300 import build

    build.build()
    L = tf.load_library()
    for name in declared_symbols():
        assert hasattr(L, name), name


def test_status_strings_without_gpu():
    L = tf.load_library()
    assert L.tf_status_string(tf.ERR_ZERO_NODE).decode().startswith("level set")
    assert L.tf_status_string(tf.OK).decode() == "ok"


def test_no_silent_fallback_without_gpu():
    """Without a usable GPU the product path raises instead of computing on the CPU."""
    import ctypes

    L = tf.load_library()
    n = ctypes.c_int(0)
    try:
        cudart = ctypes.CDLL("libcudart.so")
        have = cudart.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        have = False
    if have:
        pytest.skip("a GPU is present")
    with pytest.raises(tf.TraceFEMError):
        tf.TraceFEM()
