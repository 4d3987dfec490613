"""FP64-storage form with double-word FP32 contractions (hd_adv_set_arithmetic
FP32X2) against the CPU oracle: the same 1e-12 relative bar (max-norm,
relative to the oracle's max-norm) as native FP64, per apply and after LSRK
steps, on the parity configurations, Dirichlet/skew faces and the 6D k=3 mesh."""
import math
import zlib

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402

from test_gpu_parity import CONFIGS, _id, make, rel_err  # noqa: E402

if torch.cuda.is_available():
    from hyperdeal_gb300 import advection as A  # noqa: E402

X2_TOL = 1e-12


def make_x2(*args, **kw):
    op, prob = make(*args, **kw)
    op.set_arithmetic("fp32x2")
    assert op.arithmetic == "fp32x2"
    return op, prob


@pytest.mark.parametrize("cfg", CONFIGS, ids=[_id(c) for c in CONFIGS])
def test_apply_matches_oracle(cfg):
    dim_x, dim_v, degree, cells, vel = cfg
    D = dim_x + dim_v
    rng = np.random.default_rng(zlib.crc32(_id(cfg).encode()))
    lo = list(rng.uniform(-1, 0, D))
    hi = [l + rng.uniform(0.5, 2.0) for l in lo]
    op, prob = make_x2(dim_x, dim_v, degree, cells, vel, lo, hi)
    u = rng.standard_normal(prob.n_dofs)
    ref = O.apply(prob, u)
    src = torch.tensor(u, dtype=torch.float64, device="cuda")
    dst = op.initialize_dof_vector()
    op.apply(dst, src, 0.0)
    assert rel_err(dst.cpu().numpy(), ref) <= X2_TOL


@pytest.mark.parametrize("skew", [0.0, 0.5])
def test_apply_dirichlet_and_skew(skew):
    bc = dict(kind=2, amp=1.0, omega=[2 * math.pi] * 4, speed=[1.0, 0.15, -0.05, 0.0], cosine=[0, 1, 1, 1])
    op, prob = make_x2(2, 2, 3, [3, 2, 4, 2], [1.0, 0.15, -0.05, 0.0], lo=[-1.0] * 4, hi=[1.0] * 4,
                       periodic=(False, False), skew=skew, bc=bc)
    u = np.random.default_rng(7).standard_normal(prob.n_dofs)
    for t in (0.0, 0.37):
        dst = op.initialize_dof_vector()
        op.apply(dst, torch.tensor(u, device="cuda"), t)
        assert rel_err(dst.cpu().numpy(), O.apply(prob, u, t)) <= X2_TOL


def test_smooth_data_and_zero_values():
    """Smooth data (the contractions cancel) with exact zeros and tiny values
    mixed in (the split's zero and FP32-precision ranges below 2^-103)."""
    op, prob = make_x2(2, 2, 4, [3, 3, 2, 2], [0.9, -0.6, 0.3, 0.2])
    f = O.make_func(2, 1.0, omega=[2 * math.pi] * 4, speed=[0.0] * 4)
    u = O.interpolate(prob, f)
    u[::7] = 0.0
    u[3::11] *= 1e-35
    dst = op.initialize_dof_vector()
    op.apply(dst, torch.tensor(u, device="cuda"), 0.0)
    assert rel_err(dst.cpu().numpy(), O.apply(prob, u)) <= X2_TOL


@pytest.mark.parametrize("rk", ["rk45", "rk59"])
@pytest.mark.parametrize("fused", [True, False])
def test_lsrk_steps_match_oracle(rk, fused):
    bc = dict(kind=2, amp=1.0, omega=[2 * math.pi] * 3, speed=[1.0, 0.15, -0.05], cosine=[0, 1, 1])
    op, prob = make_x2(2, 1, 3, [3, 4, 3], [1.0, 0.15, -0.05], lo=[-1.0] * 3, hi=[1.0] * 3,
                       periodic=(False, True), bc=bc)
    u = O.interpolate(prob, O.make_func(**bc), 0.0)
    sol = torch.tensor(u, device="cuda")
    Ki, Ti = op.initialize_dof_vector(), op.initialize_dof_vector()
    integ = A.LowStorageRungeKuttaIntegrator(Ki, Ti, rk, True, fused=fused)
    dt = 0.01
    uo = u.copy()
    for s in range(3):
        integ.perform_time_step(sol, s * dt, dt, op)
        O.lsrk_step(prob, rk, uo, s * dt, dt)
    assert rel_err(sol.cpu().numpy(), uo) <= X2_TOL


def test_6d_k3_steps_match_oracle():
    """The benchmark's operator (6D, k = 3, periodic) on a small mesh: two rk45 steps."""
    vel = [1.0, 0.8, 0.6, 0.4, 0.3, 0.2]
    op, prob = make_x2(3, 3, 3, [2, 3, 2, 2, 2, 3], vel)
    u = np.random.default_rng(11).standard_normal(prob.n_dofs)
    sol = torch.tensor(u, device="cuda")
    Ki, Ti = op.initialize_dof_vector(), op.initialize_dof_vector()
    integ = A.LowStorageRungeKuttaIntegrator(Ki, Ti, "rk45")
    dt = 0.2 * op.critical_time_step() / 3 ** 1.5
    uo = u.copy()
    for s in range(2):
        integ.perform_time_step(sol, s * dt, dt, op)
        O.lsrk_step(prob, "rk45", uo, s * dt, dt)
    assert rel_err(sol.cpu().numpy(), uo) <= X2_TOL


def test_native_and_fp32x2_switch_on_one_operator():
    op, prob = make(2, 2, 3, [2, 3, 2, 2], [1.0, 0.7, 0.5, 0.3])
    assert op.arithmetic == "native"
    u = torch.randn(prob.n_dofs, dtype=torch.float64, device="cuda")
    a, b = op.initialize_dof_vector(), op.initialize_dof_vector()
    op.apply(a, u, 0.0)
    op.set_arithmetic("fp32x2")
    op.apply(b, u, 0.0)
    op.set_arithmetic("native")
    c = op.initialize_dof_vector()
    op.apply(c, u, 0.0)
    assert torch.equal(a, c)
    assert rel_err(b.cpu().numpy(), a.cpu().numpy()) <= X2_TOL


def test_fp32x2_needs_f64_collocation():
    op32, _ = make(2, 2, 3, [2, 2, 2, 2], [1.0, 0.7, 0.5, 0.3], dtype="f32")
    with pytest.raises(Exception):
        op32.set_arithmetic("fp32x2")
    assert op32.arithmetic == "native"


def test_tiles_and_autotune_keep_results():
    """The FP32x2 kernel's result does not depend on its tile: every tile of a 5D k=2 mesh and
    the autotuned one give the same bits as the default tile."""
    op, prob = make_x2(3, 2, 2, [3, 2, 2, 3, 2], [0.9, -0.4, 0.6, 0.2, -0.7])
    u = torch.randn(prob.n_dofs, dtype=torch.float64, device="cuda")
    ref = op.initialize_dof_vector()
    op.apply(ref, u, 0.0)
    max_cpb, _ = op.tile_limits()
    for cpb in sorted({1, 2, max_cpb // 2, max_cpb} - {0}):
        op.set_tile(cpb, 0)
        d = op.initialize_dof_vector()
        op.apply(d, u, 0.0)
        assert torch.equal(d, ref), cpb
    op.set_tile(0, 0)
    scratch = op.initialize_dof_vector()
    tuned = op.autotune(u, scratch, reps=1)
    assert tuned["cells_per_cta"] >= 1
    d = op.initialize_dof_vector()
    op.apply(d, u, 0.0)
    assert torch.equal(d, ref)
