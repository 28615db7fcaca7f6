"""The C-ABI library loads, exports every declared entry point, and validates
arguments on the host (no GPU needed for any of these)."""

import ctypes
import re
from pathlib import Path

import pytest

from jax_bssn_gb300 import _native

HEADERS = sorted((Path(__file__).resolve().parent.parent / "include").glob("*.h"))


def declared_functions():
    names = []
    for header in HEADERS:
        text = header.read_text()
        names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s+(bssn_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(native):
    names = declared_functions()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(native, n)]
    assert not missing, missing


def test_abi_version(native):
    assert native.bssn_abi_version() == 2


def test_workspace_sizes(native):
    p = _native.BssnParams()
    p.dx, p.dt = 0.1, 0.01
    shape = _native.Shape3(16, 16, 16)
    rhs = native.bssn_workspace_bytes(_native.OP_RHS, shape, ctypes.byref(p))
    rk4 = native.bssn_workspace_bytes(_native.OP_RK4, shape, ctypes.byref(p))
    assert rhs == (2 * 21 + 33) * 24 ** 3 * 8
    assert rk4 == (4 * 21 + 33) * 24 ** 3 * 8
    p.kappa = 0.1
    assert native.bssn_workspace_bytes(_native.OP_RHS, shape, ctypes.byref(p)) > rhs


def _fields(n):
    bufs = [(ctypes.c_double * n)() for _ in range(7)]
    f = _native.BssnFields()
    for (name, _), b in zip(_native.BssnFields._fields_, bufs):
        setattr(f, name, ctypes.cast(b, ctypes.c_void_p))
    return f, bufs


def _params(**kw):
    p = _native.BssnParams()
    p.dx, p.dt, p.mad_q = 0.1, 0.01, 1.0
    for f in range(6):
        p.owned_faces[f] = 1
    for d in range(3):
        p.owned_shape[d] = -1
        p.reduced_axes[d] = -1
    for k, v in kw.items():
        setattr(p, k, v)
    return p


@pytest.mark.parametrize("bad", [dict(dx=-1.0), dict(dx=float("nan")), dict(gauge=3)])
def test_invalid_parameters_rejected_on_host(native, bad):
    fin, _a = _fields(8 ** 3)
    fout, _b = _fields(8 ** 3)
    p = _params(**bad)
    status = native.bssn_rhs(ctypes.byref(fin), ctypes.byref(fout), _native.Shape3(8, 8, 8), ctypes.byref(p),
                             None, None, 0, None)
    assert status == _native.BSSN_ERR_INVALID
    assert native.bssn_last_error()


def test_sommerfeld_axis_needs_eight_samples(native):
    fin, _a = _fields(6 * 10 * 10)
    fout, _b = _fields(6 * 10 * 10)
    p = _params()
    p.bc[0] = 1
    status = native.bssn_rhs(ctypes.byref(fin), ctypes.byref(fout), _native.Shape3(6, 10, 10), ctypes.byref(p),
                             None, None, 0, None)
    assert status == _native.BSSN_ERR_INVALID
    assert b"eight" in native.bssn_last_error()


def test_missing_workspace_rejected(native):
    fin, _a = _fields(8 ** 3)
    fout, _b = _fields(8 ** 3)
    p = _params()
    status = native.bssn_rhs(ctypes.byref(fin), ctypes.byref(fout), _native.Shape3(8, 8, 8), ctypes.byref(p),
                             None, None, 0, None)
    assert status == _native.BSSN_ERR_WORKSPACE


def test_check_raises_value_error():
    with pytest.raises(ValueError):
        _native.check(_native.BSSN_ERR_INVALID, "unit")
    with pytest.raises(RuntimeError):
        _native.check(_native.BSSN_ERR_CUDA, "unit")
