"""CPU-only checks of the drop-in boundary: libiqsg.so loads, exports every entry point
include/iqsg.h declares, and refuses to run without a GPU instead of falling back."""
import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import REPO, gpu_available

HEADER = REPO / "include" / "iqsg.h"


def declared_symbols():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(iqsg_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def built_lib():
    import iqsg_build as _build
    return _build.build()


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert len(syms) >= 30
    for s in ("iqsg_create", "iqsg_apply_1q", "iqsg_apply_controlled_1q", "iqsg_apply_2q", "iqsg_apply_swaplike",
              "iqsg_apply_diag_2q", "iqsg_permute", "iqsg_probability", "iqsg_expectation_pauli"):
        assert s in syms


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(str(built_lib))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, f"libiqsg.so lacks {missing}"
    nm = subprocess.run(["nm", "-D", "--defined-only", str(built_lib)], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (iqsg_\w+)", nm))
    assert set(declared_symbols()) <= exported


def test_python_binding_covers_header(built_lib):
    from iqs_gb300 import _lib
    assert set(declared_symbols()) == set(_lib.SIGNATURES)


def test_errors_without_device_are_loud(built_lib):
    """No CUDA device here: creating a register must fail with an error, never fall back."""
    if gpu_available():
        pytest.skip("a GPU is present")
    import iqs_gb300
    with pytest.raises((iqs_gb300.IqsgError, MemoryError)):
        iqs_gb300.QubitRegister(4, "base", 0)
    msg = iqs_gb300.lib.iqsg_last_error().decode()
    assert msg


def test_argument_validation_is_host_side(built_lib):
    """Bad arguments are rejected before any device work: null handles and null outputs."""
    from iqs_gb300 import _lib
    lib = _lib.lib
    assert lib.iqsg_apply_1q(None, 0, None) == _lib.IQSG_EINVAL
    assert lib.iqsg_norm2(None, None) == _lib.IQSG_EINVAL
    out = ctypes.c_void_p()
    assert lib.iqsg_create(0, 0, None, ctypes.byref(out)) == _lib.IQSG_EINVAL
    assert lib.iqsg_create(41, 0, None, ctypes.byref(out)) == _lib.IQSG_EINVAL
    assert lib.iqsg_create(4, 7, None, ctypes.byref(out)) == _lib.IQSG_EINVAL
    assert lib.iqsg_create_from_device(4, 0, ctypes.c_void_p(8), None, ctypes.byref(out)) == _lib.IQSG_EINVAL
    assert lib.iqsg_destroy(None) == _lib.IQSG_OK
    assert "null" in lib.iqsg_last_error().decode() or "aligned" in lib.iqsg_last_error().decode()


def test_product_does_not_reference_oracle():
    """The shipped package and kernels never import or link the oracle."""
    for p in list((REPO / "intel-qs_gb300").rglob("*.py")) + list((REPO / "intel-qs_gb300" / "csrc").glob("*")):
        text = p.read_text(errors="ignore")
        assert "import oracle" not in text and "liboracle" not in text and "iqs_oracle" not in text, p
