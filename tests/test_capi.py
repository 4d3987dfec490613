"""C ABI checks that need no GPU: the library loads, exports every symbol the
header declares, validates descriptors before touching CUDA, and carries the
reference's LSRK tables."""
import ctypes
import os
import re

import numpy as np
import pytest

from hyperdeal_gb300 import _lib
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "hyperdeal_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hd_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def L():
    return _lib.load()


def test_every_declared_symbol_is_exported(L):
    syms = declared_symbols()
    assert len(syms) >= 16
    for s in syms:
        assert hasattr(L, s), s
    assert sorted(_lib.EXPORTED_SYMBOLS) == syms


def test_version(L):
    assert b"sm_103a" in L.hd_version()


def _desc(**kw):
    d = _lib.hd_adv_desc()
    d.dim_x, d.dim_v, d.degree, d.n_points, d.dtype = 2, 2, 3, 4, _lib.HD_F64
    for i in range(3):
        d.cells_x[i] = d.cells_v[i] = 4
        d.lo_x[i] = d.lo_v[i] = 0.0
        d.hi_x[i] = d.hi_v[i] = 1.0
    d.periodic_x = d.periodic_v = 1
    for k, v in kw.items():
        setattr(d, k, v)
    return d


@pytest.mark.parametrize("kw,code,msg", [
    (dict(dim_x=0), _lib.HD_ERR_INVALID, "dim_x"),
    (dict(dim_v=4), _lib.HD_ERR_INVALID, "dim_x"),
    (dict(degree=0, n_points=1), _lib.HD_ERR_UNSUPPORTED, "degree"),
    (dict(degree=6, n_points=7), _lib.HD_ERR_UNSUPPORTED, "degree"),
    (dict(n_points=5), _lib.HD_ERR_UNSUPPORTED, "n_points"),
    (dict(dtype=7), _lib.HD_ERR_INVALID, "dtype"),
    (dict(bc_kind=9), _lib.HD_ERR_INVALID, "bc_kind"),
    (dict(skew=float("nan")), _lib.HD_ERR_INVALID, "skew"),
])
def test_invalid_descriptor(L, kw, code, msg):
    h = ctypes.c_void_p()
    d = _desc(**kw)
    rc = L.hd_adv_create(ctypes.byref(d), ctypes.byref(h))
    assert rc == code
    assert msg in _lib.last_error()
    assert not h.value


def test_invalid_mesh(L):
    h = ctypes.c_void_p()
    d = _desc()
    d.cells_v[1] = 0
    assert L.hd_adv_create(ctypes.byref(d), ctypes.byref(h)) == _lib.HD_ERR_INVALID
    d = _desc()
    d.hi_x[0] = d.lo_x[0]
    assert L.hd_adv_create(ctypes.byref(d), ctypes.byref(h)) == _lib.HD_ERR_INVALID
    assert L.hd_adv_create(None, ctypes.byref(h)) == _lib.HD_ERR_INVALID


def test_unsupported_cell_size(L):
    # 6D degree 4 in FP64: a cell (5^6 values) does not fit in shared memory
    h = ctypes.c_void_p()
    d = _desc(dim_x=3, dim_v=3, degree=4, n_points=5)
    assert L.hd_adv_create(ctypes.byref(d), ctypes.byref(h)) == _lib.HD_ERR_UNSUPPORTED
    assert "shared memory" in _lib.last_error()


@pytest.mark.parametrize("rk", ["rk33", "rk45", "rk47", "rk59"])
def test_lsrk_tables_match_reference(L, rk):
    h = ctypes.c_void_p()
    assert L.hd_lsrk_create(rk.encode(), ctypes.byref(h)) == 0
    try:
        ns = L.hd_lsrk_n_stages(h)
        a, b = O.lsrk_coefficients(rk)
        assert ns == len(b)
        ai = (ctypes.c_double * 16)()
        bi = (ctypes.c_double * 16)()
        ci = (ctypes.c_double * 16)()
        assert L.hd_lsrk_coefficients(h, ai, bi, ci) == 0
        assert list(ai)[:ns - 1] == list(a) and list(bi)[:ns] == list(b)
        # c_s = sum_{j<s-1} b_j + a_{s-1}  (time_integrators.templates.h:172-183)
        c = [0.0] + [sum(b[:s - 1]) + a[s - 1] for s in range(1, ns)]
        assert np.allclose(list(ci)[:ns], c, rtol=0, atol=1e-15)
    finally:
        L.hd_lsrk_destroy(h)


def test_lsrk_unknown_type(L):
    h = ctypes.c_void_p()
    assert L.hd_lsrk_create(b"rk99", ctypes.byref(h)) == _lib.HD_ERR_UNSUPPORTED
    assert "rk99" in _lib.last_error()


def test_null_arguments(L):
    assert L.hd_adv_apply(None, None, None, 0.0, None) == _lib.HD_ERR_INVALID
    assert L.hd_lsrk_step(None, None, None, None, None, 0.0, 0.0, None) == _lib.HD_ERR_INVALID
    assert L.hd_lsrk_stage_update(3, 10, 1.0, 1.0, ctypes.c_void_p(16), ctypes.c_void_p(16), None,
                                  None) == _lib.HD_ERR_INVALID
    assert L.hd_adv_n_dofs(None) == -1
