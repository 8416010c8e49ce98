"""The C ABI boundary, checked without a GPU: the library builds for sm_103a,
loads, and exports every function include/qrdm_gb300.h declares; the Python
``QRDM`` mirror has the reference module's functions and arities
(QRDM_wrapper.c:131-139).  No compute call is made here."""
import ctypes
import inspect
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "qrdm_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_]+\s*\*?\s*([a-z_0-9]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_reference_entry_points():
    names = declared_functions()
    for n in ("dgeqrdm", "dgeqp3", "qrdm_dgeqrf", "qrdm_dormqr", "dgeqrdm_dev", "dgeqrdm_ex"):
        assert n in names, n


def test_library_exports_every_declared_symbol():
    from qrdm_gb300.build import build

    path = build()
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    from qrdm_gb300._lib import SIGNATURES

    assert set(SIGNATURES) >= set(declared_functions())


def test_version_string_without_gpu():
    from qrdm_gb300 import lib

    assert b"sm_103a" in lib().qrdm_version()


def test_python_module_mirrors_reference_surface():
    from qrdm_gb300 import QRDM

    arity = {"init": 0, "QRF": 6, "QP3": 7, "QRDM": 10, "DORMQR": 9}
    for name, n in arity.items():
        f = getattr(QRDM, name)
        assert len(inspect.signature(f).parameters) == n, name


def test_python_module_rejects_wrong_dtypes():
    import numpy as np
    import pytest

    from qrdm_gb300 import QRDM

    A = np.zeros((4, 3), order="F")
    with pytest.raises(TypeError):
        QRDM.QRDM(102, 4, 3, A, 4, np.zeros(3, np.int64), np.zeros(3), np.zeros(3, np.int32),
                  np.array([0.9, 0.15]), 2)
    with pytest.raises(ValueError):
        QRDM.QRDM(102, 4, 3, A[:2], 4, np.zeros(3, np.int32), np.zeros(3),
                  np.zeros(3, np.int32), np.array([0.9, 0.15]), 2)
