"""The GPU path against the layout fixtures of tests/test_layout_goldens.py, through the C ABI.

* The velocity moment of the Vlasov-Poisson path (the kernel behind
  VlasovPoissonOperation.solve_field / fields) reproduces the reference's
  ordered dumps vector_tools_02 (1+1D) and vector_tools_03 (2+2D, hierarchical
  cells mapped to lexicographic ones) entry by entry: the GPU reads the DoF
  layout exactly as the reference writes it.
* The face-trace property of tests/matrix_free/fefaceevalutation_02 for every
  (dim_x, dim_v) in {1,2,3}^2 on every kernel that reads neighbour faces: the
  generic kernel (FP64, FP32, FP32x2 arithmetic), the Gauss-quadrature kernel
  and the TMA-pipelined 3x+3v kernel, whose x2 / v0 / v1 faces are TMA boxes
  and whose v2 face is a bulk copy.
"""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402
from test_layout_goldens import (GOLD, SPLITS, face_property_cells, face_property_expected,  # noqa: E402
                                 hierarchical, linear_coordinate, printed_equal, vt03_problem, vt03_values)

if torch.cuda.is_available():
    from hyperdeal_gb300 import advection as A  # noqa: E402
    from hyperdeal_gb300 import vlasov_poisson as V  # noqa: E402


def gpu_rho(dim, cells_x, cells_v, lo, hi, values, dtype="f64"):
    p = V.VlasovPoissonParameters(dim, 3, [cells_x] * dim, [cells_v] * dim, [lo] * dim, [hi] * dim, [lo] * dim,
                                  [hi] * dim, dtype=dtype, cg_tol=1e-10, guess="zero", cg_rhs_relative=True)
    op = V.VlasovPoissonOperation(p)
    f = op.initialize_dof_vector()
    f.copy_(torch.tensor(values, dtype=f.dtype))
    op.solve_field(f)
    rho, _, _ = op.fields()
    return rho.cpu().numpy()


@pytest.mark.parametrize("refs", [2, 3, 4, 5])
def test_vector_tools_02_velocity_moment_on_gpu(refs):
    c = 2 ** refs
    prob = O.Problem(1, 1, 3, [c, c], [0.0, 0.0], [1.0, 1.0], [1.0, 1.0])
    f = O.make_func(2, 1.0, omega=[math.pi, math.pi], speed=[0.0, 0.0], cosine=[0, 1])
    u = O.interpolate(prob, f)
    for entry in GOLD["vector_tools_02"]:
        if entry["refinements"] != refs:
            continue
        if entry["function"] == "zero":
            vals = np.zeros_like(u)
        elif entry["function"] == "one":
            vals = np.ones_like(u)
        else:
            vals = u
        rho = gpu_rho(1, c, c, 0.0, 1.0, vals)
        assert len(rho) == len(entry["vec_x"])
        for ours, ref in zip(rho, entry["vec_x"]):
            assert printed_equal(ours, ref), (entry["function"], ours, ref)
        ref_oracle = O.velocity_moment(prob, vals)
        assert np.abs(rho - ref_oracle).max() <= 1e-13 * max(1.0, np.abs(ref_oracle).max())


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_vector_tools_03_velocity_moment_on_gpu(dtype):
    g = GOLD["vector_tools_03"]
    prob, c = vt03_problem()
    u = vt03_values(prob)
    rho = gpu_rho(2, c, c, g["lo"], g["hi"], u, dtype)
    ref_oracle = O.velocity_moment(prob, u.astype(np.float32).astype(np.float64) if dtype == "f32" else u)
    assert np.abs(rho - ref_oracle).max() <= 1e-13 * np.abs(ref_oracle).max()
    if dtype == "f64":
        ordered = hierarchical(rho, c, 2, 16)
        for ours, ref in zip(ordered, g["vec_x"]):
            assert printed_equal(ours, ref), (ours, ref)


def _face_property_gpu(dim_x, dim_v, dtype, quadrature="gauss_lobatto", arithmetic="native", kernel="auto"):
    D = dim_x + dim_v
    cells = face_property_cells(dim_x, dim_v)
    hi = [1.0 + 0.5 * d for d in range(D)]
    worst = 0.0
    for direction in range(D):
        prob = O.Problem(dim_x, dim_v, 3, cells, [0.0] * D, hi, [1.0] * D)
        u = linear_coordinate(prob, direction)
        for e in range(D):
            vel = [0.0] * D
            vel[e] = 1.0
            p = A.AdvectionParameters(dim_x, dim_v, 3, cells[:dim_x], cells[dim_x:], [0.0] * dim_x, hi[:dim_x],
                                      [0.0] * dim_v, hi[dim_x:], vel, dtype=dtype, quadrature=quadrature)
            op = A.AdvectionOperation(p)
            if arithmetic != "native":
                op.set_arithmetic(arithmetic)
            if kernel != "auto":
                op.set_kernel(kernel)
                assert op.kernel == kernel
            src = torch.tensor(u, dtype=op.dtype, device="cuda")
            dst = op.initialize_dof_vector()
            op.apply(dst, src, 0.0)
            if kernel == "pipelined":
                assert op.device_status() == 0
            r = dst.double().cpu().numpy()
            worst = max(worst, face_property_expected(prob, direction, e, r, quadrature == "gauss_lobatto"))
    return worst


@pytest.mark.parametrize("dim_x,dim_v", SPLITS)
@pytest.mark.parametrize("dtype,tol", [("f64", 1e-11), ("f32", 5e-4)])
def test_face_trace_property_generic_kernel(dim_x, dim_v, dtype, tol):
    assert _face_property_gpu(dim_x, dim_v, dtype, kernel="generic") < tol


@pytest.mark.parametrize("dim_x,dim_v", SPLITS)
def test_face_trace_property_fp32x2_and_gauss(dim_x, dim_v):
    assert _face_property_gpu(dim_x, dim_v, "f64", arithmetic="fp32x2") < 1e-11
    assert _face_property_gpu(dim_x, dim_v, "f64", quadrature="gauss") < 1e-11


def test_face_trace_property_pipelined_kernel():
    """3x+3v FP32 on a fully periodic 2^6 mesh: the TMA face boxes (x2, v0, v1) and the bulk-copied
    v2 face, the x0 face carried in registers along a row and the x1 face loaded one cell ahead."""
    assert _face_property_gpu(3, 3, "f32", kernel="pipelined") < 5e-4
