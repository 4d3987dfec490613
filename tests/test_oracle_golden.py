"""Pins the CPU oracle to the reference's own golden outputs (no GPU).

The fixture tests/golden/reference_goldens.json holds the reference's test
outputs (extracted by tests/golden/make_goldens.py):
  * examples/advection/tests/*.out  -- advection application time series,
    compared the way the reference's ctest does (numdiff -a 1e-5 -r 1e-8);
  * tests/time_discretization/time_integrators_0{1,2} -- LSRK stage counts and
    the rk45 known answer 118.127 for y' = y sin^2 t;
  * tests/vector_tools/vector_tools_01 -- interpolation + L2 norm/error.
"""
import json
import math
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))
CASES = GOLD["advection"]


def numdiff_equal(a, b, abs_tol=1e-5, rel_tol=1e-8):
    """numdiff semantics: equal when within the absolute OR the relative tolerance."""
    d = abs(a - b)
    return d <= abs_tol or d <= rel_tol * max(abs(a), abs(b))


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_advection_application_golden(case):
    if case["n_points"] != case["degree"] + 1:
        pytest.skip("over-integration (n_points = degree + 2) is outside the collocation hot path")
    rows = O.run_hyperrectangle(case["dim_x"], case["dim_v"], case["degree"], case["subdivisions"],
                                periodic=case["periodic_x"], collocation=case["collocation"], rk=case["rk"],
                                final_time=case["final_time"], time_step=case["time_step"], cfl=case["cfl"],
                                tick=case["tick"], skew=case["skew"])
    ref = case["rows"]
    assert len(rows) == len(ref)
    worst = 0.0
    for (t, n, e), (rt, rn, re_) in zip(rows, ref):
        # the printed time has 4 significant digits
        assert abs(t - rt) <= 0.5e-3 * max(abs(rt), 1e-3) + 1e-12
        assert numdiff_equal(n, rn), (t, n, rn)
        assert numdiff_equal(e, re_), (t, e, re_)
        worst = max(worst, abs(n - rn) / abs(rn))
    # the restatement agrees far inside the numdiff bound (printed precision is ~1e-11)
    assert worst < 1e-9


def test_lsrk_stage_counts():
    assert [len(O.lsrk_coefficients(t)[1]) for t in ("rk33", "rk45", "rk47", "rk59")] == \
        GOLD["time_integrators_01_stages"]


def test_lsrk_known_answer_rk45():
    """tests/time_discretization/time_integrators_02.cc:101-125: y' = y sin^2(t), y0 = 1, dt = 0.1, 100 steps."""
    y = np.ones(9)

    def op(src, dst, t):
        dst[:] = src * math.sin(t) ** 2

    for it in range(100):
        O.lsrk_step_op("rk45", y, 0.1 * it, 0.1, op)
    for v, ref in zip(y, GOLD["time_integrators_02_rk45_values"]):
        assert numdiff_equal(v, ref, abs_tol=1e-3)  # golden printed with 6 digits
    exact = math.exp((10 - math.sin(10) * math.cos(10)) / 2)
    assert abs(y[0] - exact) / exact < 2e-6


def test_vector_tools_01():
    """tests/vector_tools/vector_tools_01.cc:60-132: zero / one / sin(pi x) cos(pi v) on [0,1]^2, Gauss points."""
    rows = []
    for refs in range(2, 6):
        n = 2 ** refs
        p = O.Problem(1, 1, 3, [n, n], [0.0, 0.0], [1.0, 1.0], [1.0, 1.0], collocation=False)
        for f in (O.make_func(0), O.make_func(1, 1.0), O.make_func(2, 1.0, omega=[math.pi] * 2, cosine=[0, 1])):
            u = O.interpolate(p, f)
            rows.append(O.norm_and_error(p, f, 0.0, u))
    ref = GOLD["vector_tools_01_rows"]
    assert len(rows) == len(ref)
    for (a, b), (ra, rb) in zip(rows, ref):
        assert numdiff_equal(a, ra) and numdiff_equal(b, rb)
        if rb > 1e-12:
            assert abs(b - rb) / rb < 1e-5  # golden printed with 6 digits


def test_gauss_lobatto_rules():
    for n in range(2, 8):
        x, w = O.gauss_lobatto(n)
        assert x[0] == 0.0 and x[-1] == 1.0 and abs(w.sum() - 1.0) < 1e-15
        # exact for polynomials of degree 2n-3
        for p in range(2 * n - 2):
            assert abs((w * x ** p).sum() - 1.0 / (p + 1)) < 1e-14
        xg, wg = O.gauss(n)
        for p in range(2 * n):
            assert abs((wg * xg ** p).sum() - 1.0 / (p + 1)) < 1e-14


def test_oracle_collocation_conservation_and_linearity():
    """Periodic collocation operator: sum_i JxW_i (A u)_i = 0 and A is linear."""
    p = O.Problem(2, 1, 3, [3, 2, 4], [0, 0, -1], [1, 1, 1], [0.7, -0.4, 1.3])
    rng = np.random.default_rng(1)
    u = rng.standard_normal(p.n_dofs)
    v = rng.standard_normal(p.n_dofs)
    Au, Av = O.apply(p, u), O.apply(p, v)
    Auv = O.apply(p, 2.0 * u - 3.0 * v)
    assert np.allclose(Auv, 2 * Au - 3 * Av, rtol=1e-12, atol=1e-12 * np.abs(Au).max())
    x, w = O.gauss_lobatto(4)
    h = [1 / 3, 1 / 2, 2 / 4]
    jxw = np.einsum("i,j,k->kji", w * h[0], w * h[1], w * h[2]).ravel()
    mass = (Au.reshape(-1, 64) * jxw).sum()
    assert abs(mass) < 1e-12 * np.abs(Au).max()


@pytest.mark.parametrize("case", GOLD["vlasov_poisson"], ids=[c["name"] for c in GOLD["vlasov_poisson"]])
def test_vlasov_poisson_application_golden(case):
    """examples/vlasov_poisson/tests/*.out: the oracle's Vlasov-Poisson (moments, SIPG Poisson + CG,
    field, phase-space advection, rk45) against the reference's diagnostics time series."""
    rows, st = O.run_vp_hyperrectangle(case["dim_x"], case["dim_v"], case["degree"], case["cells_x"],
                                       case["cells_v"], collocation=case["collocation"],
                                       final_time=case["final_time"], time_step=case["time_step"],
                                       cfl=case["cfl"])
    ref = case["rows"]
    assert len(rows) == len(ref)
    dx = case["dim_x"]
    for r, g in zip(rows, ref):
        assert abs(r[0] - g[0]) <= 1e-3
        got = list(r[1:1 + dx]) + list(r[1 + dx:])
        exp = g[1:]
        for a, b in zip(got, exp):
            assert numdiff_equal(a, b), (r[0], a, b)
        # mass, L2 norm and kinetic energy far inside the numdiff bound
        for a, b in zip(got[dx:dx + 3], exp[dx:dx + 3]):
            assert abs(a - b) <= 1e-12 * abs(b)
        # field energy: the reference solves Poisson to a 1e-4 relative residual with multigrid
        if g[1] > 1e-6:
            assert abs(got[0] - g[1]) <= 1e-7 * g[1]


def test_poisson_sipg_operator_properties():
    """SIPG matrix: symmetric, positive semi-definite, constants in its kernel (periodic mesh)."""
    p = O.Problem(2, 2, 3, [3, 4, 2, 2], [0, 0, -6, -6], [4 * math.pi, 4 * math.pi, 6, 6], [1.0] * 4)
    n = O.x_dofs(p)
    A = np.stack([O.poisson_apply(p, np.eye(n)[i]) for i in range(n)], axis=1)
    assert np.abs(A - A.T).max() <= 1e-12 * np.abs(A).max()
    ev = np.linalg.eigvalsh(0.5 * (A + A.T))
    assert ev.min() > -1e-10 * ev.max()
    assert np.abs(O.poisson_apply(p, np.ones(n))).max() < 1e-12
