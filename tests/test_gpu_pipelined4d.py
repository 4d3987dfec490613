"""The TMA-pipelined kernel on 2x+2v degree-3 FP32 meshes with 16 cells along x0.

One x0-row of 16 cells (4,096 values) is the kernel's unit there, laid out
like one 6D cell: the x0 upwind trace is a cell of the same unit (including
the periodic wrap), the x1 trace of the neighbouring unit is read one unit
ahead, the v0 and v1 traces are TMA boxes of the neighbouring units.  Checked
through the C ABI against the oracle and the generic kernel (both velocity
signs in every direction), over fused rk45 steps, with the face-trace
property of tests/matrix_free/fefaceevalutation_02, and for the bounded-wait
time-out; meshes that do not qualify keep the generic kernel.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402
from test_layout_goldens import face_property_expected, linear_coordinate  # noqa: E402

if torch.cuda.is_available():
    from hyperdeal_gb300 import advection as A  # noqa: E402

MESHES = {
    # name: (cells x0 x1 | v0 v1, velocity)
    "mixed_signs": ([16, 2, 2, 3], [0.7, -0.5, 0.4, -0.3]),
    "positive": ([16, 3, 2, 2], [1.0, 0.8, 0.6, 0.4]),
    "negative_x0": ([16, 2, 3, 2], [-0.9, 0.5, -0.6, 0.2]),
}


def _params(cells, vel, dtype="f32"):
    hi = [1.0 + 0.25 * d for d in range(4)]
    return A.AdvectionParameters(2, 2, 3, cells[:2], cells[2:], [0.0] * 2, hi[:2], [0.0] * 2, hi[2:], vel,
                                 dtype=dtype)


def _pair(name):
    cells, vel = MESHES[name]
    op = A.AdvectionOperation(_params(cells, vel))
    gen = A.AdvectionOperation(_params(cells, vel))
    gen.set_kernel("generic")
    return op, gen


def _rel(a, b):
    return float((a.double() - b.double()).abs().max() / b.double().abs().max())


@pytest.mark.parametrize("name", sorted(MESHES))
def test_apply_matches_oracle_and_generic_kernel(name):
    op, gen = _pair(name)
    assert op.kernel == "pipelined" and gen.kernel == "generic"
    cells, vel = MESHES[name]
    hi = [1.0 + 0.25 * d for d in range(4)]
    prob = O.Problem(2, 2, 3, cells, [0.0] * 4, hi, vel)
    u = np.random.default_rng(11).standard_normal(op.n_dofs).astype(np.float32)
    src = torch.tensor(u, device="cuda")
    dst, ref = op.initialize_dof_vector(), gen.initialize_dof_vector()
    op.apply(dst, src, 0.0)
    gen.apply(ref, src, 0.0)
    assert op.device_status() == 0
    orc = torch.tensor(O.apply(prob, u.astype(np.float64)))
    assert _rel(dst.cpu(), orc) <= 2e-5
    assert _rel(dst, ref) <= 2e-6


@pytest.mark.parametrize("name", sorted(MESHES))
def test_fused_steps_match_the_generic_kernel(name):
    op, gen = _pair(name)
    u = torch.randn(op.n_dofs, device="cuda", generator=torch.Generator(device="cuda").manual_seed(4))
    dt = 0.2 * op.critical_time_step() / 3 ** 1.5
    sols = []
    for o in (op, gen):
        sol = u.clone()
        it = A.LowStorageRungeKuttaIntegrator(o.initialize_dof_vector(), o.initialize_dof_vector(), "rk45")
        for s in range(3):
            it.perform_time_step(sol, s * dt, dt, o)
        sols.append(sol)
    assert op.device_status() == 0
    assert _rel(sols[0], sols[1]) <= 5e-6


def test_face_trace_property_pipelined_2x2v():
    """u = x_dir with the velocity along e only: no jump on any face unless the pairing of the
    neighbour's face nodes is wrong (0 for e != dir, -1 for e == dir away from the wrap)."""
    cells = [16, 2, 2, 2]
    hi = [1.0 + 0.5 * d for d in range(4)]
    worst = 0.0
    for direction in range(4):
        prob = O.Problem(2, 2, 3, cells, [0.0] * 4, hi, [1.0] * 4)
        u = linear_coordinate(prob, direction)
        for e in range(4):
            vel = [0.0] * 4
            vel[e] = 1.0
            p = A.AdvectionParameters(2, 2, 3, cells[:2], cells[2:], [0.0] * 2, hi[:2], [0.0] * 2, hi[2:], vel,
                                      dtype="f32")
            op = A.AdvectionOperation(p)
            assert op.kernel == "pipelined"
            dst = op.initialize_dof_vector()
            op.apply(dst, torch.tensor(u, dtype=torch.float32, device="cuda"), 0.0)
            assert op.device_status() == 0
            r = dst.double().cpu().numpy()
            worst = max(worst, face_property_expected(prob, direction, e, r, True))
    assert worst < 5e-4, worst


def test_meshes_that_do_not_qualify_keep_the_generic_kernel():
    vel = [0.7, -0.5, 0.4, -0.3]
    assert A.AdvectionOperation(_params([8, 2, 2, 2], vel)).kernel == "generic"
    assert A.AdvectionOperation(_params([16, 2, 2, 2], vel, dtype="f64")).kernel == "generic"
    p = _params([16, 2, 2, 2], vel)
    p.periodic_v = False
    assert A.AdvectionOperation(p).kernel == "generic"


def test_bounded_wait_runs_out_and_the_operator_recovers():
    op, _ = _pair("mixed_signs")
    src = torch.randn(op.n_dofs, device="cuda", generator=torch.Generator(device="cuda").manual_seed(2))
    ref = op.initialize_dof_vector()
    op.apply(ref, src, 0.0)
    assert op.device_status() == 0
    op.set_wait_test(1 << 14, 0)  # nothing issued for the launch's first unit
    dst = torch.full_like(ref, float("nan"))
    op.apply(dst, src, 0.0)
    assert op.device_status() in (1, 2)
    assert torch.isnan(dst).any()
    op.set_wait_test(0, -1)
    dst2 = op.initialize_dof_vector()
    op.apply(dst2, src, 0.0)
    assert op.device_status() == 0
    assert torch.equal(dst2, ref)
