"""Batched uneven instances (hd_batch_*): one persistent launch per class and
stage, CUDA-graph replay, autotuned tiles.  Every instance must equal its own
single-operator path bit for bit (same cell arithmetic, only the CTA
traversal differs), and the FP64 instances the oracle."""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402

if torch.cuda.is_available():
    from hyperdeal_gb300 import advection as A  # noqa: E402
    from hyperdeal_gb300 import batch as B  # noqa: E402


# (dim_x, dim_v, degree, cells_x, cells_v, dtype, dirichlet)
SPECS = [
    (2, 2, 2, 3, 4, "f32", False),
    (2, 2, 2, 5, 3, "f32", False),   # same class as the first: one launch for both
    (2, 2, 3, 3, 3, "f64", False),
    (2, 2, 5, 2, 2, "f64", True),    # inhomogeneous Dirichlet, time-dependent data
    (2, 3, 2, 2, 3, "f32", False),
    (3, 2, 3, 2, 2, "f64", False),
    (2, 3, 4, 2, 2, "f32", True),
    (1, 1, 3, 8, 8, "f64", False),   # class without a batch kernel: launched per instance
    (3, 3, 3, 2, 2, "f32", False),   # 6D k=3 FP32 periodic: the pipelined kernel
]


def _make(spec, seed):
    dx, dv, k, cx, cv, dtype, dirichlet = spec
    D = dx + dv
    rng = np.random.default_rng(seed)
    vel = rng.standard_normal(D)
    vel /= np.linalg.norm(vel)
    bc = A.Function(2, 0.5, omega=[2 * math.pi] * D, speed=list(vel), phase=list(rng.uniform(0, 1, D))) \
        if dirichlet else None
    p = A.AdvectionParameters(dx, dv, k, [cx] * dx, [cv] * dv, [0.0] * dx, [1.0] * dx, [-1.0] * dv, [1.0] * dv,
                              list(vel), periodic_x=not dirichlet, periodic_v=not dirichlet, dtype=dtype, boundary=bc)
    op = A.AdvectionOperation(p)
    g = torch.Generator(device="cuda").manual_seed(seed)
    u = torch.randn(op.n_dofs, device="cuda", dtype=op.dtype, generator=g)
    prob = None
    if dtype == "f64":
        lo = [0.0] * dx + [-1.0] * dv
        hi = [1.0] * D
        bcf = O.make_func(2, 0.5, omega=[2 * math.pi] * D, speed=list(vel), phase=list(bc.phase)) if dirichlet else None
        prob = O.Problem(dx, dv, k, [cx] * dx + [cv] * dv, lo, hi, list(vel), periodic_x=not dirichlet,
                         periodic_v=not dirichlet, bc_func=bcf)
    return op, u, prob


def _setup():
    ops, us, probs = [], [], []
    for i, s in enumerate(SPECS):
        op, u, prob = _make(s, 100 + i)
        ops.append(op)
        us.append(u)
        probs.append(prob)
    return ops, us, probs


def test_classes_and_apply_equal_single_operators():
    ops, us, probs = _setup()
    batch = B.AdvectionBatch(ops)
    cls = batch.classes
    assert sum(c["members"] for c in cls) == len(ops)
    by_key = {(c["dim"], c["degree"], c["dtype"]): c for c in cls}
    assert by_key[(4, 2, "f32")]["members"] == 2 and by_key[(4, 2, "f32")]["batched"]
    assert not by_key[(2, 3, "f64")]["batched"] and not by_key[(6, 3, "f32")]["batched"]
    dst = [op.initialize_dof_vector() for op in ops]
    times = [0.1 * i for i in range(len(ops))]
    batch.apply(dst, us, times)
    for op, u, d, t, prob in zip(ops, us, dst, times, probs):
        ref = op.initialize_dof_vector()
        op.apply(ref, u, t)
        assert torch.equal(d, ref)
        if prob is not None:
            o = O.apply(prob, u.cpu().numpy(), t)
            assert np.abs(d.cpu().numpy() - o).max() <= 1e-12 * np.abs(o).max()


@pytest.mark.parametrize("rk", ["rk45", "rk33"])
def test_steps_equal_single_operators(rk):
    ops, us, _ = _setup()
    batch = B.AdvectionBatch(ops, rk)
    sols = [u.clone() for u in us]
    Ks = [op.initialize_dof_vector() for op in ops]
    Ts = [op.initialize_dof_vector() for op in ops]
    refs = [u.clone() for u in us]
    rK = [op.initialize_dof_vector() for op in ops]
    rT = [op.initialize_dof_vector() for op in ops]
    integ = [A.LowStorageRungeKuttaIntegrator(k, t, rk) for k, t in zip(rK, rT)]
    dts = [0.01 * (1 + i % 3) for i in range(len(ops))]
    times = [0.0] * len(ops)
    for step in range(3):
        batch.perform_time_step(sols, Ks, Ts, times, dts)
        for i, op in enumerate(ops):
            integ[i].perform_time_step(refs[i], times[i], dts[i], op)
        times = [t + d for t, d in zip(times, dts)]
    for s, r in zip(sols, refs):
        assert torch.equal(s, r)


def test_graph_replay_equals_steps():
    ops, us, _ = _setup()
    ops_g = ops
    batch = B.AdvectionBatch(ops_g)
    sols = [u.clone() for u in us]
    Ks = [op.initialize_dof_vector() for op in ops_g]
    Ts = [op.initialize_dof_vector() for op in ops_g]
    dts = [0.005 * (1 + i % 2) for i in range(len(ops_g))]
    t0 = [0.0] * len(ops_g)
    batch.capture_graph(sols, Ks, Ts, t0, dts)
    for _ in range(3):
        batch.replay_graph()
    torch.cuda.synchronize()
    # reference: six plain batch steps from the same data
    batch2 = B.AdvectionBatch(ops_g)
    refs = [u.clone() for u in us]
    rK = [op.initialize_dof_vector() for op in ops_g]
    rT = [op.initialize_dof_vector() for op in ops_g]
    times = list(t0)
    for _ in range(6):
        batch2.perform_time_step(refs, rK, rT, times, dts)
        times = [t + d for t, d in zip(times, dts)]
    for spec, s, r in zip(SPECS, sols, refs):
        if spec[-1]:
            # time-dependent boundary data: the replayed stage times advance on
            # the device (t_s + 2 dt per replay) and round differently from the
            # host's running sum, so the boundary values differ at round-off
            assert (s - r).abs().max() <= 1e-12 * r.abs().max()
        else:
            assert torch.equal(s, r)


def test_autotune_keeps_results():
    ops, us, _ = _setup()
    batch = B.AdvectionBatch(ops)
    dst = [op.initialize_dof_vector() for op in ops]
    before = [op.initialize_dof_vector() for op in ops]
    batch.apply(before, us)
    classes = batch.autotune(us, dst, reps=2)
    assert all(c["cells_per_cta"] >= 1 for c in classes if c["batched"])
    batch.apply(dst, us)
    for a, b in zip(dst, before):
        assert torch.equal(a, b)
    # every tile gives the same result
    for i, c in enumerate(batch.classes):
        if c["batched"]:
            batch.set_tile(i, 1, 1)
    batch.apply(dst, us)
    for a, b in zip(dst, before):
        assert torch.equal(a, b)


def test_bad_arguments():
    ops, us, _ = _setup()
    batch = B.AdvectionBatch(ops)
    with pytest.raises(A.HdError):
        batch.apply(us[:-1], us[:-1])
    with pytest.raises(A.HdError):
        batch.apply(us, us)  # dst == src
    with pytest.raises(A.HdError):
        batch.replay_graph()  # nothing recorded


def test_single_operator_autotune_keeps_results():
    ops, us, _ = _setup()
    for op, u in zip(ops[:3], us[:3]):
        ref = op.initialize_dof_vector()
        op.apply(ref, u, 0.0)
        dst = op.initialize_dof_vector()
        tile = op.autotune(u, dst, reps=2)
        assert tile["cells_per_cta"] >= 1 and tile["ms_per_apply"] > 0
        op.apply(dst, u, 0.0)
        assert torch.equal(dst, ref)


def test_fp32x2_instances_equal_single_operators():
    """FP64 operators switched to FP32x2 arithmetic form their own batch class
    (beside the native FP64 ones of the same shape) and equal their own
    single-operator FP32x2 path bit for bit, apply and fused steps."""
    specs = [(2, 2, 3, 3, 3, "f64", False), (2, 2, 3, 2, 4, "f64", False), (2, 3, 2, 2, 3, "f64", True),
             (2, 2, 3, 3, 2, "f64", False)]
    ops, us, probs = [], [], []
    for i, s in enumerate(specs):
        op, u, prob = _make(s, 300 + i)
        if i < 3:
            op.set_arithmetic("fp32x2")
        ops.append(op)
        us.append(u)
        probs.append(prob)
    batch = B.AdvectionBatch(ops, "rk45")
    cls = batch.classes
    x2 = [c for c in cls if c["arithmetic"] == "fp32x2"]
    nat = [c for c in cls if c["arithmetic"] == "native"]
    assert sum(c["members"] for c in x2) == 3 and all(c["batched"] for c in x2)
    assert len(nat) == 1 and nat[0]["members"] == 1 and (nat[0]["dim"], nat[0]["degree"]) == (4, 3)
    dst = [op.initialize_dof_vector() for op in ops]
    batch.apply(dst, us, [0.2] * len(ops))
    for op, u, d, prob in zip(ops, us, dst, probs):
        ref = op.initialize_dof_vector()
        op.apply(ref, u, 0.2)
        assert torch.equal(d, ref)
        o = O.apply(prob, u.cpu().numpy(), 0.2)
        assert np.abs(d.cpu().numpy() - o).max() <= 1e-12 * np.abs(o).max()
    sols = [u.clone() for u in us]
    Ks = [op.initialize_dof_vector() for op in ops]
    Ts = [op.initialize_dof_vector() for op in ops]
    refs = [u.clone() for u in us]
    integ = [A.LowStorageRungeKuttaIntegrator(op.initialize_dof_vector(), op.initialize_dof_vector(), "rk45")
             for op in ops]
    times, dts = [0.0] * len(ops), [0.01] * len(ops)
    for step in range(2):
        batch.perform_time_step(sols, Ks, Ts, times, dts)
        for i, op in enumerate(ops):
            integ[i].perform_time_step(refs[i], times[i], dts[i], op)
        times = [t + d for t, d in zip(times, dts)]
    for s, r in zip(sols, refs):
        assert torch.equal(s, r)
