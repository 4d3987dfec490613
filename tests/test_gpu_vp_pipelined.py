"""The TMA-pipelined Vlasov-Poisson advection (hd_vp_pipe.cuh): FP32, 2x+2v, degree 3,
collocation, 16 cells along x0.

The unit is one x0-row of 16 cells; both neighbours' traces along every
direction are at hand, and every line takes its upwind side from the sign of
its own velocity (v at the line's v-node for the x-directions, grad phi at
its x-node for the v-directions), so the field's sign changes inside a unit
are exercised by any perturbed Maxwellian.  Checked through the C ABI against
the generic kernel and the oracle, over fused rk45 steps, and for the
bounded-wait time-out; other meshes keep the generic kernel.
"""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402

if torch.cuda.is_available():
    from hyperdeal_gb300 import vlasov_poisson as V  # noqa: E402


def _op(cells_x=(16, 2), cells_v=(4, 3), dtype="f32", kernel="auto"):
    p = V.VlasovPoissonParameters(2, 3, list(cells_x), list(cells_v), [0.0] * 2, [4 * math.pi] * 2, [-6.0] * 2,
                                  [6.0] * 2, dtype=dtype, cg_tol=1e-12, guess="zero")
    op = V.VlasovPoissonOperation(p)
    if kernel != "auto":
        op.set_kernel(kernel)
    return op


def _prob(cells_x=(16, 2), cells_v=(4, 3)):
    return O.Problem(2, 2, 3, list(cells_x) + list(cells_v), [0.0, 0.0, -6.0, -6.0], [4 * math.pi] * 2 + [6.0] * 2,
                     [1.0, 1.0, 6.0, 6.0], collocation=True)


def _f0(prob, seed=3):
    fo = O.interpolate(prob, O.vp_initial_function(2, 2, eps=0.2, perturbed_dims=(0, 1)))
    fo = fo * (1.0 + 0.05 * np.random.default_rng(seed).standard_normal(fo.size))
    return fo.astype(np.float32)


def _rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_apply_matches_generic_kernel_and_oracle():
    pipe, gen = _op(), _op(kernel="generic")
    assert pipe.kernel == "pipelined" and gen.kernel == "generic"
    prob = _prob()
    fo = _f0(prob)
    src = torch.tensor(fo, device="cuda")
    d1, d2 = pipe.initialize_dof_vector(), gen.initialize_dof_vector()
    pipe.apply(d1, src, 0.0)
    gen.apply(d2, src, 0.0)
    assert pipe.device_status() == 0
    assert _rel(d1.cpu().numpy(), d2.cpu().numpy()) <= 1e-6
    st = O.VPState(prob, 1e-12)
    ref = np.zeros(fo.size)
    st.operator(fo.astype(np.float64), ref, 0.0)
    assert _rel(d1.cpu().numpy(), ref) <= 2e-5


def test_fused_steps_match_the_generic_kernel():
    out = {}
    for kernel in ("auto", "generic"):
        op = _op(kernel=kernel)
        f = op.initialize_dof_vector()
        op.interpolate(V.perturbed_maxwellian(2, eps=0.05, perturbed_dims=(0, 1)), f)
        Ki, Ti = op.initialize_dof_vector(), op.initialize_dof_vector()
        integ = V.LowStorageRungeKuttaIntegrator(Ki, Ti, "rk45")
        for s in range(3):
            op.perform_time_step(integ, f, s * 2e-3, 2e-3)
        out[kernel] = (f.double().cpu().numpy(), op.diagnostics(f))
        if kernel == "auto":
            assert op.kernel == "pipelined" and op.device_status() == 0
    assert _rel(out["auto"][0], out["generic"][0]) <= 5e-6
    assert _rel(out["auto"][1], out["generic"][1]) <= 1e-5


def test_bounded_wait_runs_out_and_the_operator_recovers():
    op = _op()
    prob = _prob()
    src = torch.tensor(_f0(prob), device="cuda")
    ref = op.initialize_dof_vector()
    op.apply(ref, src, 0.0)
    assert op.device_status() == 0
    op.set_wait_test(1 << 14, 0)  # nothing issued for unit 0: its consumers' wait runs out
    dst = torch.full_like(ref, float("nan"))
    op.apply(dst, src, 0.0)
    assert op.device_status() in (1, 2)
    assert torch.isnan(dst).any()
    op.set_wait_test(0, -1)
    dst2 = op.initialize_dof_vector()
    op.apply(dst2, src, 0.0)
    assert op.device_status() == 0
    assert torch.equal(dst2, ref)


def test_meshes_that_do_not_qualify_keep_the_generic_kernel():
    assert _op(cells_x=(8, 2)).kernel == "generic"
    assert _op(dtype="f64").kernel == "generic"
    with pytest.raises(V.HdError):
        _op(dtype="f64", kernel="pipelined")
    with pytest.raises(V.HdError):
        _op().set_wait_test(0, 3)
