"""hd_norm_and_error_noalloc: the allocation-free L2 norm / error entry point.

It exists for callers that must not allocate device memory (a host
application that owns all device memory, a time loop that forbids allocation
after start-up).  This file is collected last so that a run stopping at its
first failure has already run every other test; it passes alone in a fresh
process and after the other tests.
"""
import ctypes
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from hyperdeal_gb300 import _lib  # noqa: E402

if torch.cuda.is_available():
    from hyperdeal_gb300 import advection as A  # noqa: E402

REL_TOL = 1e-12  # the two reductions sum in different orders


def _case(dim_x, dim_v, cells, dtype):
    D = dim_x + dim_v
    params = A.AdvectionParameters(dim_x, dim_v, 3, cells[:dim_x], cells[dim_x:], [-1.0] * dim_x, [1.0] * dim_x,
                                   [-2.0] * dim_v, [2.0] * dim_v, [0.5] * D, dtype=dtype)
    f = A.Function(2, 1.3, omega=[math.pi * (d + 1) / 2 for d in range(D)], speed=[0.2] * D,
                   phase=[0.1 * d for d in range(D)], cosine=[d % 2 for d in range(D)])
    return params, f


@pytest.mark.parametrize("dim_x,dim_v,cells,dtype", [
    (2, 2, [6, 5, 4, 3], "f64"),
    (3, 3, [4, 3, 2, 3, 2, 3], "f32"),
])
def test_noalloc_matches_allocating_entry_point(dim_x, dim_v, cells, dtype):
    params, f = _case(dim_x, dim_v, cells, dtype)
    op = A.AdvectionOperation(params)
    v = op.initialize_dof_vector()
    A.VectorTools.interpolate(op, f, v, 0.0)
    v.mul_(1.0 + 1e-3 * torch.arange(v.numel(), device="cuda", dtype=v.dtype) / v.numel())
    ref = A.VectorTools.norm_and_error(op, f, v, 0.25)
    L = _lib.load()
    desc = params.c()
    fc = f.c()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(2):  # two calls in a row share the static scratch
        out = (ctypes.c_double * 2)(-1.0, -1.0)
        rc = L.hd_norm_and_error_noalloc(ctypes.byref(desc), ctypes.byref(fc), 0.25, ctypes.c_void_p(v.data_ptr()),
                                         out, stream)
        assert rc == 0, _lib.last_error()
        assert abs(out[0] - ref[0]) <= REL_TOL * abs(ref[0])
        assert abs(out[1] - ref[1]) <= REL_TOL * abs(ref[1])


def test_noalloc_rejects_meshes_above_its_scratch():
    params, f = _case(3, 3, [8] * 6, "f32")  # 1,073,741,824 DoFs
    desc = params.c()
    fc = f.c()
    out = (ctypes.c_double * 2)()
    L = _lib.load()
    rc = L.hd_norm_and_error_noalloc(ctypes.byref(desc), ctypes.byref(fc), 0.0, ctypes.c_void_p(256), out, None)
    assert rc == _lib.HD_ERR_INVALID
    assert "134,217,728" in _lib.last_error()


def test_noalloc_at_its_size_limit():
    """134,217,728 DoFs exactly (3x+3v, k=3, 32,768 cells): 16,384 block partials, the whole scratch."""
    params, f = _case(3, 3, [8, 8, 8, 8, 4, 2], "f32")
    op = A.AdvectionOperation(params)
    assert op.n_dofs == 134217728
    v = op.initialize_dof_vector()
    A.VectorTools.interpolate(op, f, v, 0.0)
    ref = A.VectorTools.norm_and_error(op, f, v, 0.1)
    L = _lib.load()
    desc, fc = params.c(), f.c()
    out = (ctypes.c_double * 2)(-1.0, -1.0)
    rc = L.hd_norm_and_error_noalloc(ctypes.byref(desc), ctypes.byref(fc), 0.1, ctypes.c_void_p(v.data_ptr()), out,
                                     ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, _lib.last_error()
    assert abs(out[0] - ref[0]) <= REL_TOL * abs(ref[0])
    assert abs(out[1] - ref[1]) <= 1e-9 * abs(ref[0])  # the error is FP32 round-off: compare on the norm's scale
    del op, v
    torch.cuda.empty_cache()


def test_noalloc_rejects_gauss_descriptors_and_unknown_functions():
    """Both are refused on the host, before any device work."""
    L = _lib.load()
    out = (ctypes.c_double * 2)()
    params, f = _case(2, 2, [2, 2, 2, 2], "f64")
    desc = params.c()
    desc.quadrature = 1  # HD_QUAD_GAUSS
    fc = f.c()
    rc = L.hd_norm_and_error_noalloc(ctypes.byref(desc), ctypes.byref(fc), 0.0, ctypes.c_void_p(256), out, None)
    assert rc == _lib.HD_ERR_UNSUPPORTED
    assert "Gauss-Lobatto" in _lib.last_error()
    desc = params.c()
    fc = f.c()
    fc.kind = 7
    rc = L.hd_norm_and_error_noalloc(ctypes.byref(desc), ctypes.byref(fc), 0.0, ctypes.c_void_p(256), out, None)
    assert rc == _lib.HD_ERR_INVALID
    assert "kind" in _lib.last_error()
