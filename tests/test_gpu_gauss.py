"""Gauss-quadrature (non-collocation) ECL path on the GPU against the oracle's
Gauss branch, and the reference's Gauss goldens reproduced end to end."""
import json
import math
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402

if torch.cuda.is_available():
    from hyperdeal_gb300 import advection as A  # noqa: E402

F64_TOL = 1e-12
F32_TOL = 2e-6


def make(dim_x, dim_v, degree, cells, velocity, lo=None, hi=None, periodic=(True, True), skew=0.0, dtype="f64",
         bc=None):
    D = dim_x + dim_v
    lo = lo or [0.0] * D
    hi = hi or [1.0] * D
    params = A.AdvectionParameters(dim_x, dim_v, degree, cells[:dim_x], cells[dim_x:], lo[:dim_x], hi[:dim_x],
                                   lo[dim_x:], hi[dim_x:], velocity, periodic_x=periodic[0], periodic_v=periodic[1],
                                   skew=skew, dtype=dtype, boundary=None if bc is None else A.Function(**bc),
                                   quadrature="gauss")
    prob = O.Problem(dim_x, dim_v, degree, list(cells), lo, hi, velocity, periodic_x=periodic[0],
                     periodic_v=periodic[1], skew=skew, collocation=False,
                     bc_func=None if bc is None else O.make_func(**bc))
    return A.AdvectionOperation(params), prob


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


CONFIGS = [
    (1, 1, 3, [5, 4], [1.0, 0.5]),
    (1, 1, 1, [3, 7], [-0.3, 0.9]),
    (1, 2, 2, [3, 4, 2], [0.4, -1.1, 0.0]),
    (2, 1, 4, [2, 3, 3], [-0.6, 0.2, 0.8]),
    (2, 2, 3, [3, 4, 2, 3], [1.0, 0.7, -0.5, 0.3]),
    (2, 3, 2, [2, 2, 3, 2, 2], [0.1, 0.2, 0.3, -0.4, 0.5]),
    (3, 3, 2, [2, 2, 2, 2, 2, 3], [1.0, 0.8, -0.6, 0.4, 0.3, -0.2]),
    (3, 3, 3, [2, 2, 1, 2, 2, 2], [1.0, -0.8, 0.6, 0.4, 0.0, -0.2]),
]


@pytest.mark.parametrize("cfg", CONFIGS, ids=lambda c: "%dx%dv_k%d" % c[:3])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_apply_matches_oracle_gauss(cfg, dtype):
    dx, dv, k, cells, vel = cfg
    op, prob = make(dx, dv, k, cells, vel, dtype=dtype)
    rng = np.random.default_rng(sum(cells) + k)
    u = rng.standard_normal(prob.n_dofs)
    if dtype == "f32":
        u = u.astype(np.float32).astype(np.float64)
    src = torch.tensor(u, dtype=op.dtype, device="cuda")
    dst = op.initialize_dof_vector()
    op.apply(dst, src, 0.0)
    ref = O.apply(prob, u, 0.0)
    assert rel_err(dst.double().cpu().numpy(), ref) <= (F64_TOL if dtype == "f64" else F32_TOL)


@pytest.mark.parametrize("skew", [0.0, 0.5])
def test_gauss_dirichlet_and_skew(skew):
    bc = dict(kind=2, amp=0.7, omega=[2 * math.pi] * 4, speed=[1.0, 0.15, -0.05, 0.0], phase=[0.1, 0.2, 0.3, 0.4],
              cosine=[0, 1, 1, 1])
    op, prob = make(2, 2, 3, [3, 2, 2, 3], [1.0, -0.15, -0.05, 0.3], lo=[-1.0] * 4, hi=[1.0] * 4,
                    periodic=(False, False), skew=skew, bc=bc)
    rng = np.random.default_rng(5)
    u = rng.standard_normal(prob.n_dofs)
    dst = op.initialize_dof_vector()
    op.apply(dst, torch.tensor(u, device="cuda"), 0.37)
    ref = O.apply(prob, u, 0.37)
    assert rel_err(dst.cpu().numpy(), ref) <= F64_TOL


@pytest.mark.parametrize("fused", [True, False])
def test_gauss_lsrk_steps(fused):
    op, prob = make(2, 2, 2, [3, 3, 2, 2], [0.7, -0.4, 0.3, 0.9])
    rng = np.random.default_rng(9)
    u = rng.standard_normal(prob.n_dofs)
    sol = torch.tensor(u, device="cuda")
    Ki, Ti = op.initialize_dof_vector(), op.initialize_dof_vector()
    integ = A.LowStorageRungeKuttaIntegrator(Ki, Ti, "rk45", fused=fused)
    uo = u.copy()
    dt = 0.01
    for s in range(3):
        integ.perform_time_step(sol, s * dt, dt, op)
        O.lsrk_step(prob, "rk45", uo, s * dt, dt)
    assert rel_err(sol.cpu().numpy(), uo) <= F64_TOL


def test_gauss_norm_and_error():
    op, prob = make(2, 2, 3, [3, 2, 2, 3], [1.0, 0.5, 0.2, 0.1])
    f = dict(kind=2, amp=1.3, omega=[2 * math.pi] * 4, speed=[1.0, 0.5, 0.2, 0.1], phase=[0.0, 0.3, 0.1, 0.2],
             cosine=[0, 1, 1, 0])
    fo = O.make_func(**f)
    u = O.interpolate(prob, fo, 0.0) * 1.01
    n, e = A.VectorTools.norm_and_error(op, A.Function(**f), torch.tensor(u, device="cuda"), 0.2)
    rn, re_ = O.norm_and_error(prob, fo, 0.2, u)
    assert abs(n - rn) / rn < 1e-13 and abs(e - re_) / re_ < 1e-11


def _gauss_goldens():
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))
    return [c for c in gold["advection"] if not c["collocation"] and c["n_points"] == c["degree"] + 1]


@pytest.mark.parametrize("case", _gauss_goldens(), ids=lambda c: c["name"])
def test_gauss_golden_on_gpu(case):
    """The reference's Gauss-quadrature goldens (ECL and FCL outputs compute the same operator) through
    the CUDA path with the fused LSRK, norms with Gauss quadrature."""
    dx, dv, k = case["dim_x"], case["dim_v"], case["degree"]
    D = dx + dv
    adv = [1.0, 0.15, -0.05, 0.0, 0.0, 0.0][:D]
    exact = dict(kind=2, amp=1.0, omega=[2 * math.pi] * D, speed=adv, cosine=[0] + [1] * (D - 1))
    periodic = case["periodic_x"]
    op, _ = make(dx, dv, k, case["subdivisions"], adv, lo=[-1.0] * D, hi=[1.0] * D, periodic=(periodic, periodic),
                 skew=case["skew"], bc=None if periodic else exact)
    f = A.Function(**exact)
    sol = op.initialize_dof_vector()
    A.VectorTools.interpolate(op, f, sol, 0.0)
    Ki, Ti = op.initialize_dof_vector(), op.initialize_dof_vector()
    integ = A.LowStorageRungeKuttaIntegrator(Ki, Ti, case["rk"])
    dt = A.time_step_rule(case["time_step"], case["cfl"], op.critical_time_step(), k, 0.0, case["final_time"])
    rows = []

    def diag(t):
        if O.tick_due(t, 0.0, dt, case["tick"]):
            rows.append((t,) + A.VectorTools.norm_and_error(op, f, sol, t))

    A.TimeLoop(dt, 0.0, case["final_time"]).loop(sol, integ.perform_time_step, op, diag)
    assert len(rows) == len(case["rows"])
    for (t, n, e), (rt, rn, re_) in zip(rows, case["rows"]):
        assert abs(t - rt) <= 1e-3 * max(1.0, abs(rt))  # the reference prints times with 4 digits
        assert abs(n - rn) <= max(1e-5, 1e-8 * abs(rn))  # the reference's numdiff tolerances
        assert abs(e - re_) <= max(1e-5, 1e-8 * abs(re_))
