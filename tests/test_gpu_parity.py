"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Tolerances (max-norm, relative to the oracle's max-norm):
  FP64 apply / LSRK step : 1e-12   (the reference's per-apply bar)
  FP32 storage form      : 2e-6 per apply against the FP64 oracle fed the same
                           (float-rounded) input; 2e-5 after several steps
"""
import math
import zlib

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402

if torch.cuda.is_available():
    from hyperdeal_gb300 import advection as A  # noqa: E402

F64_TOL = 1e-12
F32_TOL = 2e-6


def make(dim_x, dim_v, degree, cells, velocity, lo=None, hi=None, periodic=(True, True), skew=0.0,
         dtype="f64", bc=None):
    D = dim_x + dim_v
    lo = lo or [0.0] * D
    hi = hi or [1.0] * D
    params = A.AdvectionParameters(dim_x, dim_v, degree, cells[:dim_x], cells[dim_x:], lo[:dim_x], hi[:dim_x],
                                   lo[dim_x:], hi[dim_x:], velocity, periodic_x=periodic[0],
                                   periodic_v=periodic[1], skew=skew, dtype=dtype,
                                   boundary=None if bc is None else A.Function(**bc))
    prob = O.Problem(dim_x, dim_v, degree, list(cells), lo, hi, velocity, periodic_x=periodic[0],
                     periodic_v=periodic[1], skew=skew, bc_func=None if bc is None else O.make_func(**bc))
    return A.AdvectionOperation(params), prob


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


CONFIGS = [
    # dim_x, dim_v, degree, cells, velocity
    (1, 1, 3, [5, 4], [1.0, 0.5]),
    (1, 1, 1, [3, 7], [-0.3, 0.9]),
    (1, 2, 2, [3, 4, 2], [0.4, -1.1, 0.0]),
    (2, 1, 4, [2, 3, 3], [-0.6, 0.2, 0.8]),
    (2, 2, 3, [3, 4, 2, 3], [1.0, 0.7, -0.5, 0.3]),
    (2, 2, 5, [2, 2, 3, 2], [0.3, -0.2, 0.1, 0.9]),
    (1, 3, 2, [3, 2, 2, 3], [0.5, 0.5, -0.5, 1.5]),
    (3, 2, 3, [2, 3, 2, 2, 3], [0.9, -0.4, 0.6, 0.2, -0.7]),
    (2, 3, 2, [2, 2, 3, 2, 2], [0.1, 0.2, 0.3, -0.4, 0.5]),
    (3, 3, 3, [2, 3, 2, 2, 2, 3], [1.0, 0.8, 0.6, -0.4, 0.3, 0.2]),
    (3, 3, 1, [3, 2, 2, 3, 2, 2], [1.0, -0.8, 0.6, 0.4, 0.0, -0.2]),
]


def _id(c):
    return "%dx%dv_k%d" % (c[0], c[1], c[2])


@pytest.mark.parametrize("cfg", CONFIGS, ids=[_id(c) for c in CONFIGS])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_apply_matches_oracle(cfg, dtype):
    dim_x, dim_v, degree, cells, vel = cfg
    D = dim_x + dim_v
    rng = np.random.default_rng(zlib.crc32(_id(cfg).encode()))
    lo = list(rng.uniform(-1, 0, D))
    hi = [l + rng.uniform(0.5, 2.0) for l in lo]
    op, prob = make(dim_x, dim_v, degree, cells, vel, lo, hi, dtype=dtype)
    u = rng.standard_normal(prob.n_dofs)
    if dtype == "f32":
        u = u.astype(np.float32).astype(np.float64)
    ref = O.apply(prob, u)
    src = torch.tensor(u, dtype=op.dtype, device="cuda")
    dst = op.initialize_dof_vector()
    op.apply(dst, src, 0.0)
    got = dst.double().cpu().numpy()
    assert rel_err(got, ref) <= (F64_TOL if dtype == "f64" else F32_TOL)


@pytest.mark.parametrize("bc", [None, dict(kind=2, amp=1.0, omega=[2 * math.pi] * 4, speed=[1.0, 0.15, -0.05, 0.0],
                                           cosine=[0, 1, 1, 1])])
@pytest.mark.parametrize("skew", [0.0, 0.5])
def test_apply_dirichlet_and_skew(bc, skew):
    vel = [1.0, 0.15, -0.05, 0.0]
    op, prob = make(2, 2, 3, [3, 2, 4, 2], vel, lo=[-1.0] * 4, hi=[1.0] * 4, periodic=(False, False), skew=skew,
                    bc=bc)
    rng = np.random.default_rng(7)
    u = rng.standard_normal(prob.n_dofs)
    for t in (0.0, 0.37):
        ref = O.apply(prob, u, t)
        src = torch.tensor(u, device="cuda")
        dst = op.initialize_dof_vector()
        op.apply(dst, src, t)
        assert rel_err(dst.cpu().numpy(), ref) <= F64_TOL


def test_mixed_periodicity():
    op, prob = make(1, 2, 3, [4, 3, 2], [-0.7, 0.4, -1.2], periodic=(True, False))
    u = np.random.default_rng(3).standard_normal(prob.n_dofs)
    src = torch.tensor(u, device="cuda")
    dst = op.initialize_dof_vector()
    op.apply(dst, src, 0.0)
    assert rel_err(dst.cpu().numpy(), O.apply(prob, u)) <= F64_TOL


@pytest.mark.parametrize("rk", ["rk33", "rk45", "rk47", "rk59"])
@pytest.mark.parametrize("fused", [True, False])
def test_lsrk_steps_match_oracle(rk, fused):
    bc = dict(kind=2, amp=1.0, omega=[2 * math.pi] * 3, speed=[1.0, 0.15, -0.05], cosine=[0, 1, 1])
    op, prob = make(2, 1, 3, [3, 4, 3], [1.0, 0.15, -0.05], lo=[-1.0] * 3, hi=[1.0] * 3,
                    periodic=(False, True), bc=bc)
    f = O.make_func(**bc)
    u = O.interpolate(prob, f, 0.0)
    sol = torch.tensor(u, device="cuda")
    Ki = op.initialize_dof_vector()
    Ti = op.initialize_dof_vector()
    integ = A.LowStorageRungeKuttaIntegrator(Ki, Ti, rk, True, fused=fused)
    dt = 0.01
    uo = u.copy()
    for s in range(3):
        integ.perform_time_step(sol, s * dt, dt, op)
        O.lsrk_step(prob, rk, uo, s * dt, dt)
    assert rel_err(sol.cpu().numpy(), uo) <= F64_TOL


def test_fused_equals_unfused_f32():
    op, prob = make(3, 3, 3, [2, 2, 3, 2, 3, 2], [1.0, 0.8, 0.6, 0.4, 0.3, 0.2], dtype="f32")
    u = torch.randn(prob.n_dofs, device="cuda", dtype=torch.float32)
    sols = []
    for fused in (True, False):
        sol = u.clone()
        Ki, Ti = op.initialize_dof_vector(), op.initialize_dof_vector()
        integ = A.LowStorageRungeKuttaIntegrator(Ki, Ti, "rk45", fused=fused)
        for s in range(2):
            integ.perform_time_step(sol, s * 1e-3, 1e-3, op)
        sols.append(sol.double().cpu().numpy())
    assert rel_err(sols[0], sols[1]) <= 1e-6


def test_f32_steps_against_f64_oracle():
    vel = [1.0, 0.7, 0.5, 0.3]
    op, prob = make(2, 2, 3, [4, 4, 4, 4], vel, dtype="f32")
    f = O.make_func(2, 1.0, omega=[2 * math.pi] * 4, speed=[0.0] * 4)
    u0 = O.interpolate(prob, f)
    sol = torch.tensor(u0, dtype=torch.float32, device="cuda")
    Ki, Ti = op.initialize_dof_vector(), op.initialize_dof_vector()
    integ = A.LowStorageRungeKuttaIntegrator(Ki, Ti, "rk45")
    dt = 0.2 * op.critical_time_step() / 3 ** 1.5
    uo = u0.copy()
    for s in range(10):
        integ.perform_time_step(sol, s * dt, dt, op)
        O.lsrk_step(prob, "rk45", uo, s * dt, dt)
    assert rel_err(sol.double().cpu().numpy(), uo) <= 2e-5


def test_interpolate_and_norms():
    op, prob = make(2, 2, 3, [3, 2, 2, 3], [1.0, 0.5, 0.2, 0.1], lo=[-1] * 4, hi=[1] * 4)
    fd = dict(kind=2, amp=1.3, omega=[math.pi, 2.0, 1.0, 3.0], speed=[1.0, 0.5, 0.2, 0.1], phase=[0.1, 0.2, 0.3, 0.4],
              cosine=[0, 1, 0, 1])
    f, fo = A.Function(**fd), O.make_func(**fd)
    v = op.initialize_dof_vector()
    A.VectorTools.interpolate(op, f, v, 0.3)
    ref = O.interpolate(prob, fo, 0.3)
    assert rel_err(v.cpu().numpy(), ref) <= 1e-14
    n, e = A.VectorTools.norm_and_error(op, f, v * 1.01, 0.3)
    rn, re_ = O.norm_and_error(prob, fo, 0.3, ref * 1.01)
    assert abs(n - rn) / rn < 1e-13 and abs(e - re_) / re_ < 1e-12


def test_golden_hyperrectangle_05_on_gpu():
    """The reference's golden adv_2D_2D_k3.hyperrectangle_05 (ECL + Dirichlet + collocation, rk45, T=1)
    reproduced through the CUDA path (fused LSRK)."""
    import json
    import os
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))
    case = [c for c in gold["advection"] if c["name"] == "adv_2D_2D_k3.hyperrectangle_05"][0]
    exact = dict(kind=2, amp=1.0, omega=[2 * math.pi] * 4, speed=[1.0, 0.15, -0.05, 0.0], cosine=[0, 1, 1, 1])
    op, prob = make(2, 2, 3, [4, 4, 4, 4], [1.0, 0.15, -0.05, 0.0], lo=[-1.0] * 4, hi=[1.0] * 4,
                    periodic=(False, False), bc=exact)
    f = A.Function(**exact)
    sol = op.initialize_dof_vector()
    A.VectorTools.interpolate(op, f, sol, 0.0)
    Ki, Ti = op.initialize_dof_vector(), op.initialize_dof_vector()
    integ = A.LowStorageRungeKuttaIntegrator(Ki, Ti, case["rk"])
    dt = A.time_step_rule(case["time_step"], case["cfl"], op.critical_time_step(), 3, 0.0, case["final_time"])
    rows = []

    def diag(t):
        if O.tick_due(t, 0.0, dt, case["tick"]):
            rows.append((t,) + A.VectorTools.norm_and_error(op, f, sol, t))

    A.TimeLoop(dt, 0.0, case["final_time"]).loop(sol, integ.perform_time_step, op, diag)
    assert len(rows) == len(case["rows"])
    for (t, n, e), (rt, rn, re_) in zip(rows, case["rows"]):
        assert abs(n - rn) <= max(1e-5, 1e-8 * abs(rn))
        assert abs(e - re_) <= max(1e-5, 1e-8 * abs(re_))
        assert abs(n - rn) / rn < 1e-9


def test_full_size_6d_f32_properties():
    """6D k=3, 8^3 x 8^3 cells (1.07e9 DoFs) in FP32: sampled cells against the oracle, exact translation
    equivariance along a periodic direction, and discrete mass conservation of the operator."""
    vel = [1.0, 0.8, 0.6, 0.4, 0.3, 0.2]
    op, prob = make(3, 3, 3, [8] * 6, vel, dtype="f32")
    n = op.n_dofs
    assert n == 1073741824
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    src = torch.randn(n, device="cuda", dtype=torch.float32, generator=g)
    dst = op.initialize_dof_vector()
    op.apply(dst, src, 0.0)
    cells = np.array([0, 1, 7, 8, 63, 64, 511, 512, 4095, 32768, 262143, 123456, 200001])
    host = src.cpu().numpy()
    ref = O.apply_cells(prob, host, cells)
    got = dst.view(-1, 4096)[torch.tensor(cells, device="cuda")].double().cpu().numpy()
    assert rel_err(got, ref) <= F32_TOL
    del host
    # shift the input by one cell along v1 (cell stride 8*512) -> output shifts identically (bitwise)
    s6 = src.view(8, 8, 8, 512, 4096)
    shifted = torch.roll(s6, shifts=1, dims=1).reshape(-1)
    dst2 = op.initialize_dof_vector()
    op.apply(dst2, shifted, 0.0)
    assert torch.equal(dst2.view(8, 8, 8, 512, 4096), torch.roll(dst.view(8, 8, 8, 512, 4096), 1, 1))
    del shifted, dst2, s6
    # conservation: sum_i JxW_i K_i = 0 on a periodic mesh (up to FP32 round-off)
    x, w = O.gauss_lobatto(4)
    w6 = torch.tensor(np.einsum("a,b,c,d,e,f->fedcba", w, w, w, w, w, w).ravel(), device="cuda",
                      dtype=torch.float64)
    K = dst.view(-1, 4096)
    mass = (K.double() @ w6).sum().item()
    scale = (K.double().abs() @ w6).sum().item()
    assert abs(mass) <= 1e-6 * scale


def test_full_size_6d_f64_properties():
    """6D k=3, 8^3 x 8^3 cells (1.07e9 DoFs, 8.6 GB per vector) in FP64, native and FP32x2 contractions:
    sampled cells against the oracle at the FP64 bar, exact translation equivariance along a periodic
    direction, and discrete mass conservation."""
    vel = [1.0, 0.8, 0.6, 0.4, 0.3, 0.2]
    op, prob = make(3, 3, 3, [8] * 6, vel, dtype="f64")
    n = op.n_dofs
    assert n == 1073741824
    g = torch.Generator(device="cuda")
    g.manual_seed(1)
    src = torch.randn(n, device="cuda", dtype=torch.float64, generator=g)
    cells = np.array([0, 1, 7, 8, 63, 64, 511, 512, 4095, 32768, 262143, 123456, 200001])
    idx = torch.tensor(cells, device="cuda")
    ref = O.apply_cells(prob, src.cpu().numpy(), cells)
    dst = op.initialize_dof_vector()
    for arith in ("native", "fp32x2"):
        op.set_arithmetic(arith)
        op.apply(dst, src, 0.0)
        got = dst.view(-1, 4096)[idx].cpu().numpy()
        assert rel_err(got, ref) <= F64_TOL, arith
    op.set_arithmetic("native")
    op.apply(dst, src, 0.0)
    # shift the input by one cell along v2 (the slowest direction) -> the output shifts identically
    shifted = torch.roll(src.view(8, 32768 * 4096), shifts=1, dims=0).reshape(-1)
    del src
    dst2 = op.initialize_dof_vector()
    op.apply(dst2, shifted, 0.0)
    del shifted
    assert torch.equal(dst2.view(8, -1), torch.roll(dst.view(8, -1), 1, 0))
    del dst2
    # conservation: sum_i JxW_i K_i = 0 on a periodic mesh (up to FP64 round-off)
    x, w = O.gauss_lobatto(4)
    w6 = torch.tensor(np.einsum("a,b,c,d,e,f->fedcba", w, w, w, w, w, w).ravel(), device="cuda",
                      dtype=torch.float64)
    K = dst.view(-1, 4096)
    mass = (K @ w6).sum().item()
    scale = (K.abs() @ w6).sum().item()
    assert abs(mass) <= 1e-13 * scale
    del dst, K
    torch.cuda.empty_cache()


PIPE_CASES = [
    ([2, 3, 2, 2, 2, 3], [1.0, 0.8, 0.6, 0.4, 0.3, 0.2]),
    ([3, 2, 2, 3, 2, 2], [-1.0, 0.8, -0.6, 0.4, -0.3, 0.2]),
    ([1, 2, 2, 2, 2, 1], [0.5, -0.7, 0.0, 1.2, -0.3, 0.9]),
    ([5, 1, 2, 3, 1, 2], [-0.2, 0.0, 0.6, -0.4, 0.3, -0.25]),
    ([4, 4, 4, 4, 4, 4], [1.0, 0.8, 0.6, 0.4, 0.3, 0.2]),
]


@pytest.mark.parametrize("cells,vel", PIPE_CASES, ids=["c%d" % i for i in range(len(PIPE_CASES))])
def test_pipelined_kernel_matches_oracle_and_generic(cells, vel):
    rng = np.random.default_rng(11)
    lo = list(rng.uniform(-1, 0, 6))
    hi = [l + rng.uniform(0.5, 2.0) for l in lo]
    op, prob = make(3, 3, 3, cells, vel, lo, hi, dtype="f32")
    assert op.kernel == "pipelined"
    u = rng.standard_normal(prob.n_dofs).astype(np.float32)
    src = torch.tensor(u, device="cuda")
    d_pipe = op.initialize_dof_vector()
    op.apply(d_pipe, src, 0.0)
    assert op.device_status() == 0
    op.set_kernel("generic")
    assert op.kernel == "generic"
    d_gen = op.initialize_dof_vector()
    op.apply(d_gen, src, 0.0)
    ref = O.apply(prob, u.astype(np.float64))
    assert rel_err(d_pipe.double().cpu().numpy(), ref) <= F32_TOL
    assert rel_err(d_pipe.double().cpu().numpy(), d_gen.double().cpu().numpy()) <= 1e-6
    # fused LSRK steps through both kernels
    sols = []
    for kern in ("pipelined", "generic"):
        op.set_kernel(kern)
        sol = src.clone()
        Ki, Ti = op.initialize_dof_vector(), op.initialize_dof_vector()
        integ = A.LowStorageRungeKuttaIntegrator(Ki, Ti, "rk45")
        for s in range(3):
            integ.perform_time_step(sol, s * 1e-3, 1e-3, op)
        sols.append(sol.double().cpu().numpy())
    assert op.device_status() == 0
    assert rel_err(sols[0], sols[1]) <= 1e-6
    uo = u.astype(np.float64)
    for s in range(3):
        O.lsrk_step(prob, "rk45", uo, s * 1e-3, 1e-3)
    assert rel_err(sols[0], uo) <= 2e-5


def test_pipelined_kernel_selection_rules():
    op, _ = make(3, 3, 3, [2] * 6, [1.0] * 6, dtype="f32", periodic=(True, False))
    assert op.kernel == "generic"
    with pytest.raises(A.HdError):
        op.set_kernel("pipelined")
    op64, _ = make(3, 3, 3, [2] * 6, [1.0] * 6, dtype="f64")
    assert op64.kernel == "generic"


def test_pipelined_launches_on_two_streams_overlap():
    """The pipelined kernel hands out rows from a per-launch counter (a ring of them per
    operator): steps of two independent states launched on two streams of one operator,
    overlapping on the device, give the bits of the same steps run one after the other."""
    op, prob = make(3, 3, 3, [4, 3, 4, 2, 3, 4], [1.0, 0.8, 0.6, 0.4, 0.3, 0.2], dtype="f32")
    assert op.kernel == "pipelined"
    g = torch.Generator(device="cuda").manual_seed(5)
    states = [torch.randn(prob.n_dofs, device="cuda", generator=g) for _ in range(2)]
    # reference: one after the other on the current stream
    refs = []
    for u in states:
        sol = u.clone()
        integ = A.LowStorageRungeKuttaIntegrator(op.initialize_dof_vector(), op.initialize_dof_vector(), "rk45")
        for s in range(3):
            integ.perform_time_step(sol, s * 1e-3, 1e-3, op)
        refs.append(sol.clone())
    # the same steps interleaved on two streams
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    sols = [u.clone() for u in states]
    integs = [A.LowStorageRungeKuttaIntegrator(op.initialize_dof_vector(), op.initialize_dof_vector(), "rk45")
              for _ in states]
    torch.cuda.synchronize()
    for s in range(3):
        for j in range(2):
            with torch.cuda.stream(streams[j]):
                integs[j].perform_time_step(sols[j], s * 1e-3, 1e-3, op)
    torch.cuda.synchronize()
    assert op.device_status() == 0
    for sol, ref in zip(sols, refs):
        assert torch.equal(sol, ref)
