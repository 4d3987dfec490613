"""Failure detection of the pipelined kernel without a GPU fault.

Every mbarrier wait of hd::ecl6_kernel is bounded.  A test hook
(hd_adv_set_wait_test) shortens the bound and makes the producer warp that
claims the launch's first row issue nothing for one cell of it, so the compute
warps' wait for that slot runs out: the kernel records the time-out in the operator's device status,
stops its remaining work without stores, waits (bounded) for its own copies in
flight and returns.  Nothing faults or hangs; the next launch without the hook
gives the normal results and status 0, and the stream stays usable.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if torch.cuda.is_available():
    from hyperdeal_gb300 import advection as A  # noqa: E402

VEL = [1.0, 0.8, 0.6, 0.4, 0.3, 0.2]


def _op():
    # rows of 4 cells: the CTA that claims the first row reaches cells 0..3 of it
    p = A.AdvectionParameters(3, 3, 3, [4, 2, 2], [2, 2, 2], [0.0] * 3, [1.0] * 3, [0.0] * 3, [1.0] * 3, VEL,
                              dtype="f32")
    op = A.AdvectionOperation(p)
    assert op.kernel == "pipelined"
    return op


@pytest.mark.parametrize("skip", [0, 1, 3])
def test_bounded_wait_runs_out_and_the_operator_recovers(skip):
    op = _op()
    g = torch.Generator(device="cuda").manual_seed(2)
    src = torch.randn(op.n_dofs, device="cuda", generator=g)
    ref = op.initialize_dof_vector()
    op.apply(ref, src, 0.0)
    assert op.device_status() == 0
    # a wait that runs out: ~2^14 try_wait rounds (milliseconds) instead of seconds
    op.set_wait_test(1 << 14, skip)
    dst = torch.full_like(ref, float("nan"))
    op.apply(dst, src, 0.0)
    status = op.device_status()  # synchronises: the launch returned
    assert status in (1, 2), status
    assert torch.isnan(dst).any()  # the aborted CTA stored nothing for its remaining cells
    # the hook off: normal results, status 0, the stream usable
    op.set_wait_test(0, -1)
    dst2 = op.initialize_dof_vector()
    op.apply(dst2, src, 0.0)
    assert op.device_status() == 0
    assert torch.equal(dst2, ref)
    sol, sol_ref = src.clone(), src.clone()
    it = A.LowStorageRungeKuttaIntegrator(op.initialize_dof_vector(), op.initialize_dof_vector(), "rk45")
    it_ref = A.LowStorageRungeKuttaIntegrator(op.initialize_dof_vector(), op.initialize_dof_vector(), "rk45",
                                              fused=False)
    it.perform_time_step(sol, 0.0, 1e-3, op)
    it_ref.perform_time_step(sol_ref, 0.0, 1e-3, op)
    assert op.device_status() == 0
    assert float((sol - sol_ref).abs().max() / sol_ref.abs().max()) < 1e-6
    assert float(torch.ones(4, device="cuda").sum()) == 4.0


def test_wait_test_hook_rejects_bad_values():
    op = _op()
    with pytest.raises(A.HdError):
        op.set_wait_test(0, -2)
