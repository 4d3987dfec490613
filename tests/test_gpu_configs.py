"""The benchmark configurations' own checks (synthetic data of each config's shape).

C1  1x+1v, k=3, 32x32 cells on periodic [0,1]^2, a = (1.0, 0.5), f0 = sin(2 pi x) sin(2 pi v):
    one apply + 100 rk45 steps at CFL 0.2 against the oracle and the exact translated solution.
C2  2x+2v, k=3, 16^2 x 16^2 cells, a = (1.0, 0.7, 0.5, 0.3), f0 = prod sin(2 pi coord):
    FP64 against the oracle (2 steps, 1e-12) and the FP32-storage form against FP64 after 50 steps.
C3  3x+3v, k=3, 8^3 x 8^3 cells: covered by test_gpu_parity.test_full_size_6d_f32_properties and bench.py.
"""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402

if torch.cuda.is_available():
    from hyperdeal_gb300 import advection as A  # noqa: E402


def _setup(dim_x, dim_v, cells, vel, dtype):
    D = dim_x + dim_v
    p = A.AdvectionParameters(dim_x, dim_v, 3, [cells] * dim_x, [cells] * dim_v, [0.0] * dim_x, [1.0] * dim_x,
                              [0.0] * dim_v, [1.0] * dim_v, vel, dtype=dtype)
    prob = O.Problem(dim_x, dim_v, 3, [cells] * D, [0.0] * D, [1.0] * D, vel)
    return A.AdvectionOperation(p), prob


def test_config1_2d_100_steps():
    vel = [1.0, 0.5]
    op, prob = _setup(1, 1, 32, vel, "f64")
    assert op.n_dofs == 16384
    f0 = dict(kind=2, amp=1.0, omega=[2 * math.pi] * 2, speed=[0.0, 0.0])
    u0 = O.interpolate(prob, O.make_func(**f0))
    # one apply
    src = torch.tensor(u0, device="cuda")
    dst = op.initialize_dof_vector()
    op.apply(dst, src, 0.0)
    ref = O.apply(prob, u0)
    assert np.abs(dst.cpu().numpy() - ref).max() <= 1e-12 * np.abs(ref).max()
    # 100 rk45 steps at CFL 0.2 (dt = CFL * dt_crit / k^1.5)
    dt = 0.2 * op.critical_time_step() / 3 ** 1.5
    assert abs(dt - 0.2 * (1 / 32) / 3 ** 1.5) < 1e-15
    sol = src.clone()
    Ki, Ti = op.initialize_dof_vector(), op.initialize_dof_vector()
    integ = A.LowStorageRungeKuttaIntegrator(Ki, Ti, "rk45")
    uo = u0.copy()
    for s in range(100):
        integ.perform_time_step(sol, s * dt, dt, op)
        O.lsrk_step(prob, "rk45", uo, s * dt, dt)
    got = sol.cpu().numpy()
    assert np.abs(got - uo).max() <= 1e-12 * np.abs(uo).max()
    # against the exact translated solution f0(x - a t)
    t = 100 * dt
    exact = A.Function(2, 1.0, omega=[2 * math.pi] * 2, speed=vel)
    norm, err = A.VectorTools.norm_and_error(op, exact, sol, t)
    _, err_o = O.norm_and_error(prob, O.make_func(2, 1.0, omega=[2 * math.pi] * 2, speed=vel), t, uo)
    assert abs(err - err_o) <= 1e-9 * err_o
    assert err < 1e-5 and abs(norm - 0.5) < 1e-4


def test_config2_4d_f64_vs_oracle_and_f32_vs_f64():
    vel = [1.0, 0.7, 0.5, 0.3]
    f0 = A.Function(2, 1.0, omega=[2 * math.pi] * 4, speed=[0.0] * 4)
    op64, prob = _setup(2, 2, 16, vel, "f64")
    assert op64.n_dofs == 16777216
    dt = 0.2 * op64.critical_time_step() / 3 ** 1.5
    s64 = op64.initialize_dof_vector()
    A.VectorTools.interpolate(op64, f0, s64, 0.0)
    u = s64.cpu().numpy().copy()
    K64, T64 = op64.initialize_dof_vector(), op64.initialize_dof_vector()
    i64 = A.LowStorageRungeKuttaIntegrator(K64, T64, "rk45")
    for s in range(2):
        i64.perform_time_step(s64, s * dt, dt, op64)
        O.lsrk_step(prob, "rk45", u, s * dt, dt)
    assert np.abs(s64.cpu().numpy() - u).max() <= 1e-12 * np.abs(u).max()
    # FP32 storage against FP64 after 50 steps from the same initial data
    op32, _ = _setup(2, 2, 16, vel, "f32")
    s32 = op32.initialize_dof_vector()
    A.VectorTools.interpolate(op32, f0, s32, 0.0)
    A.VectorTools.interpolate(op64, f0, s64, 0.0)
    K32, T32 = op32.initialize_dof_vector(), op32.initialize_dof_vector()
    i32 = A.LowStorageRungeKuttaIntegrator(K32, T32, "rk45")
    for s in range(50):
        i32.perform_time_step(s32, s * dt, dt, op32)
        i64.perform_time_step(s64, s * dt, dt, op64)
    rel_l2 = float(torch.linalg.vector_norm(s32.double() - s64) / torch.linalg.vector_norm(s64))
    assert rel_l2 < 2e-6, rel_l2
