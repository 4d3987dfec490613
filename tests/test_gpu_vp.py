"""Vlasov-Poisson right-hand side on the GPU (hd_vp_*) against the oracle.

Gauss-Lobatto collocation, periodic, dim_x == dim_v.  FP64 pieces that do not
involve CG (moment, Poisson right-hand side, SIPG product via the field of a
given potential, interpolation) agree to round-off; everything downstream of
CG agrees to the CG tolerance.  The learned CG initial guess is checked for
its gradients (against numpy), for leaving the converged fields unchanged,
for its fallbacks, for the CG iterations it saves and for the step time it
saves against both plain guesses.
"""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402

if torch.cuda.is_available():
    from hyperdeal_gb300 import vlasov_poisson as V  # noqa: E402


def _setup(dim_x, degree, cx, cv, dtype="f64", guess="previous", cg_tol=1e-12, rhs_relative=False,
           cg_precond="block_jacobi", learn_fit="least_squares", quadrature="gauss_lobatto", poisson_solver="cg"):
    D = 2 * dim_x
    lo = [0.0] * dim_x + [-6.0] * dim_x
    hi = [4 * math.pi] * dim_x + [6.0] * dim_x
    params = V.VlasovPoissonParameters(dim_x, degree, [cx] * dim_x, [cv] * dim_x, lo[:dim_x], hi[:dim_x],
                                       lo[dim_x:], hi[dim_x:], dtype=dtype, cg_tol=cg_tol, guess=guess,
                                       cg_rhs_relative=rhs_relative, cg_precond=cg_precond, learn_fit=learn_fit,
                                       quadrature=quadrature, poisson_solver=poisson_solver)
    prob = O.Problem(dim_x, dim_x, degree, [cx] * dim_x + [cv] * dim_x, lo, hi, [1.0] * dim_x + [6.0] * dim_x,
                     collocation=quadrature == "gauss_lobatto")
    assert len(lo) == D
    return V.VlasovPoissonOperation(params), prob


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


CASES = [(1, 3, 8, 8), (2, 3, 4, 4), (2, 2, 3, 5), (3, 2, 2, 2)]


QUADS = ["gauss_lobatto", "gauss"]


@pytest.mark.parametrize("quadrature", QUADS)
@pytest.mark.parametrize("dim_x,degree,cx,cv", CASES)
def test_interpolate_moment_rhs_field(dim_x, degree, cx, cv, quadrature):
    """With Gauss quadrature the right-hand side takes the Gauss mass matrix, the SIPG matrix the
    Gauss-point integrals, and the field lives at the Gauss points -- each against the oracle's
    non-collocation branch."""
    op, prob = _setup(dim_x, degree, cx, cv, guess="zero", quadrature=quadrature)
    f0 = V.perturbed_maxwellian(dim_x, perturbed_dims=tuple(range(dim_x)))
    f = op.initialize_dof_vector()
    op.interpolate(f0, f)
    fo = O.interpolate(prob, O.vp_initial_function(dim_x, dim_x, perturbed_dims=tuple(range(dim_x))))
    assert _rel(f.cpu().numpy(), fo) <= 1e-14
    op.solve_field(f)
    rho, phi, E = (t.cpu().numpy() for t in op.fields())
    rho_o = O.velocity_moment(prob, fo)
    assert _rel(rho, rho_o) <= 1e-13
    rhs_o = O.poisson_rhs(prob, rho_o)
    # the GPU potential solves the oracle's system to the CG tolerance
    res = O.poisson_apply(prob, phi) - rhs_o
    assert np.linalg.norm(res) <= 1e-10 * np.linalg.norm(rhs_o)
    phi_o = np.zeros_like(rho_o)
    O.poisson_solve(prob, rhs_o, phi_o, 1e-12)
    assert _rel(phi - phi.mean(), phi_o - phi_o.mean()) <= 1e-8
    # the field is the exact derivative of the GPU potential
    assert _rel(E, O.vp_field(prob, phi)) <= 1e-13
    st = op.cg_stats()
    assert st["solves"] == 1 and st["last_iterations"] > 0 and st["last_residual"] <= 1e-12


@pytest.mark.parametrize("quadrature", QUADS)
@pytest.mark.parametrize("dim_x,degree,cx,cv", CASES)
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_apply_matches_oracle(dim_x, degree, cx, cv, dtype, quadrature):
    op, prob = _setup(dim_x, degree, cx, cv, dtype=dtype, quadrature=quadrature)
    rng = np.random.default_rng(7 + dim_x * 10 + degree)
    fo = O.interpolate(prob, O.vp_initial_function(dim_x, dim_x, eps=0.2))
    fo = fo * (1.0 + 0.05 * rng.standard_normal(fo.size))
    if dtype == "f32":
        fo = fo.astype(np.float32).astype(np.float64)
    tdt = torch.float64 if dtype == "f64" else torch.float32
    src = torch.tensor(fo, dtype=tdt, device="cuda")
    dst = op.initialize_dof_vector()
    op.apply(dst, src, 0.0)
    st = O.VPState(prob, 1e-12)
    ref = np.zeros_like(fo)
    st.operator(fo, ref, 0.0)
    tol = 1e-9 if dtype == "f64" else 2e-5
    assert _rel(dst.cpu().numpy(), ref) <= tol
    # the operator is the advection with the field of f: evaluating it again gives the same result
    dst2 = op.initialize_dof_vector()
    op.apply(dst2, src, 0.0)
    assert _rel(dst2.cpu().numpy(), dst.cpu().numpy()) <= (1e-10 if dtype == "f64" else 1e-5)


@pytest.mark.parametrize("poisson_solver", ["cg", "direct"])
def test_gauss_golden_vp_2D_2D_k3_hyperrectangle_01(poisson_solver):
    """The reference's Vlasov-Poisson golden examples/vlasov_poisson/tests/vp_2D_2D_k3.hyperrectangle_01
    (2x2v, k = 3, 4 cells per direction, Gauss quadrature with k + 1 points, rk45 to t = 0.5) replayed
    on the GPU through the C ABI: every diagnostics row within numdiff's tolerances, mass, L2 norm
    and kinetic energy to 1e-12, the field energy to 1e-7 (the reference solves Poisson with
    multigrid to a 1e-4 reduction) -- with CG and with the direct solve."""
    from test_oracle_golden import GOLD, numdiff_equal
    case = GOLD["vlasov_poisson"][0]
    assert case["name"] == "vp_2D_2D_k3.hyperrectangle_01" and not case["collocation"]
    rows, op = V.run_hyperrectangle(case["dim_x"], case["degree"], case["cells_x"], case["cells_v"],
                                    final_time=case["final_time"], time_step=case["time_step"], cfl=case["cfl"],
                                    quadrature="gauss", poisson_solver=poisson_solver)
    ref = case["rows"]
    assert len(rows) == len(ref)
    dx = case["dim_x"]
    for r, g in zip(rows, ref):
        assert abs(r[0] - g[0]) <= 1e-3
        got, exp = list(r[1:]), g[1:]
        for a, b in zip(got, exp):
            assert numdiff_equal(a, b), (r[0], a, b)
        for a, b in zip(got[dx:dx + 3], exp[dx:dx + 3]):
            assert abs(a - b) <= 1e-12 * abs(b), (r[0], a, b)
        if g[1] > 1e-6:
            assert abs(got[0] - g[1]) <= 1e-7 * g[1], (r[0], got[0], g[1])


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_gauss_fused_step_equals_unfused_and_refuses_fp32x2(dtype):
    dim_x, degree, cx, cv = 2, 3, 4, 6
    out = {}
    for fused in (True, False):
        op, _ = _setup(dim_x, degree, cx, cv, dtype=dtype, guess="zero", quadrature="gauss")
        f = op.initialize_dof_vector()
        op.interpolate(V.perturbed_maxwellian(dim_x, eps=0.05, perturbed_dims=(0, 1)), f)
        Ki, Ti = op.initialize_dof_vector(), op.initialize_dof_vector()
        integ = V.LowStorageRungeKuttaIntegrator(Ki, Ti, "rk45", fused=fused)
        for s in range(3):
            op.perform_time_step(integ, f, s * 1e-3, 1e-3)
        out[fused] = f.double().cpu().numpy()
    assert _rel(out[True], out[False]) <= (1e-12 if dtype == "f64" else 2e-6)
    if dtype == "f64":
        with pytest.raises(V.HdError):
            op.set_arithmetic("fp32x2")


@pytest.mark.parametrize("quadrature", QUADS)
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_apply_matches_oracle_unequal_cells(dtype, quadrature):
    """x- and v-meshes with different cell counts per direction (the x-line velocity table is laid
    out per direction, so every v-direction's cells are found whatever the other's count)."""
    cells_x, cells_v = [3, 2], [4, 3]
    p = V.VlasovPoissonParameters(2, 3, cells_x, cells_v, [0.0] * 2, [4 * math.pi] * 2, [-6.0] * 2, [6.0] * 2,
                                  dtype=dtype, cg_tol=1e-12, guess="zero", quadrature=quadrature)
    op = V.VlasovPoissonOperation(p)
    prob = O.Problem(2, 2, 3, cells_x + cells_v, [0.0, 0.0, -6.0, -6.0], [4 * math.pi] * 2 + [6.0] * 2,
                     [1.0, 1.0, 6.0, 6.0], collocation=quadrature == "gauss_lobatto")
    fo = O.interpolate(prob, O.vp_initial_function(2, 2, eps=0.2, perturbed_dims=(0, 1)))
    fo = fo * (1.0 + 0.05 * np.random.default_rng(5).standard_normal(fo.size))
    if dtype == "f32":
        fo = fo.astype(np.float32).astype(np.float64)
    src = torch.tensor(fo, dtype=torch.float64 if dtype == "f64" else torch.float32, device="cuda")
    dst = op.initialize_dof_vector()
    op.apply(dst, src, 0.0)
    st = O.VPState(prob, 1e-12)
    ref = np.zeros_like(fo)
    st.operator(fo, ref, 0.0)
    assert _rel(dst.cpu().numpy(), ref) <= (1e-9 if dtype == "f64" else 2e-5)


def test_apply_rejects_bad_input():
    op, _ = _setup(1, 3, 4, 4)
    a = op.initialize_dof_vector()
    with pytest.raises(V.HdError):
        op.apply(a, a, 0.0)
    with pytest.raises(V.HdError):
        op.apply(a, torch.zeros(3, dtype=torch.float64, device="cuda"), 0.0)
    with pytest.raises(V.HdError):
        V.VlasovPoissonOperation(V.VlasovPoissonParameters(2, 3, [4, 4], [4, 4], [0, 0], [1, 1], [0, 0], [1, 1],
                                                           cg_tol=0.0))


@pytest.mark.parametrize("quadrature", QUADS)
@pytest.mark.parametrize("dim_x,degree,cells", [(1, 3, 8), (2, 3, 4)])
def test_time_loop_diagnostics_match_oracle(dim_x, degree, cells, quadrature):
    rows, op = V.run_hyperrectangle(dim_x, degree, cells, cells, final_time=0.05, tick=0.01, quadrature=quadrature)
    rows_o, st = O.run_vp_hyperrectangle(dim_x, dim_x, degree, cells, cells,
                                         collocation=quadrature == "gauss_lobatto", final_time=0.05, tick=0.01)
    assert len(rows) == len(rows_o) and len(rows) >= 5
    for r, ro in zip(rows, rows_o):
        assert abs(r[0] - ro[0]) <= 1e-14
        r, ro = np.array(r[1:]), np.array(ro[1:])
        scale = np.maximum(np.abs(ro), 1e-12)
        # momentum is zero up to the round-off of sums of size ~ mass * max|v|
        assert np.all(np.abs(r - ro) <= 1e-8 * scale + 1e-12), (r, ro)
    # mass is conserved by the scheme
    assert abs(rows[-1][1 + dim_x] - rows[0][1 + dim_x]) <= 1e-12 * abs(rows[0][1 + dim_x])


@pytest.mark.parametrize("n,r,B", [(200, 8, 13), (2048, 16, 10)])
def test_learn_loss_grad_matches_numpy(n, r, B):
    rng = np.random.default_rng(3)
    W1 = (rng.standard_normal((r, n)) / np.sqrt(n)).astype(np.float32)
    W2 = (rng.standard_normal((n, r)) / np.sqrt(r)).astype(np.float32)
    X = rng.standard_normal((B, n)).astype(np.float32)
    Y = rng.standard_normal((B, n)).astype(np.float32)
    loss, dW1, dW2 = V.learn_loss_grad(*(torch.tensor(a, device="cuda") for a in (W1, W2, X, Y)))
    W1d, W2d, Xd, Yd = (a.astype(np.float64) for a in (W1, W2, X, Y))
    H = Xd @ W1d.T
    Err = H @ W2d.T - Yd
    ref_loss = 0.5 / B * np.sum(Err * Err)
    ref_dW2 = Err.T @ H / B
    ref_dW1 = (Err @ W2d).T @ Xd / B
    assert abs(loss - ref_loss) <= 1e-5 * ref_loss
    assert _rel(dW2.cpu().numpy(), ref_dW2) <= 1e-4
    assert _rel(dW1.cpu().numpy(), ref_dW1) <= 1e-4
    # finite-difference check of one entry of each gradient (float64 numpy)
    def L(a, b):
        e = (Xd @ a.T) @ b.T - Yd
        return 0.5 / B * np.sum(e * e)
    h = 1e-6
    a = W1d.copy(); a[2, 5] += h
    assert abs((L(a, W2d) - ref_loss) / h - ref_dW1[2, 5]) <= 1e-4 * max(1.0, abs(ref_dW1[2, 5]))
    b = W2d.copy(); b[7, 3] += h
    assert abs((L(W1d, b) - ref_loss) / h - ref_dW2[7, 3]) <= 1e-4 * max(1.0, abs(ref_dW2[7, 3]))


def _run_steps(op, f, n_steps, dt):
    Ki, Ti = op.initialize_dof_vector(), op.initialize_dof_vector()
    integ = V.LowStorageRungeKuttaIntegrator(Ki, Ti, "rk45")
    for s in range(n_steps):
        op.perform_time_step(integ, f, s * dt, dt)
    return f


@pytest.mark.parametrize("learn_fit", ["least_squares", "adam"])
@pytest.mark.parametrize("rhs_relative", [False, True])
def test_learned_guess_same_solution(rhs_relative, learn_fit):
    """The learned guess only changes where CG starts: the fields after a number of
    steps agree with the previous-potential run to the CG tolerance, the selection
    picks the learned guess at least once, and the first solves fall back (the
    least-squares fit starts from 0 before its first pair, the Adam-trained
    network from the previous potential before its second)."""
    dim_x, degree, cx, cv = 2, 3, 4, 6
    runs = {}
    for guess in ("previous", "learned"):
        op, _ = _setup(dim_x, degree, cx, cv, guess=guess, cg_tol=1e-12, rhs_relative=rhs_relative,
                       learn_fit=learn_fit)
        f = op.initialize_dof_vector()
        op.interpolate(V.perturbed_maxwellian(dim_x, eps=0.05, perturbed_dims=(0, 1)), f)
        hx, hv = 4 * math.pi / cx, 12.0 / cv
        dt = 0.05 * min(hx, hv / 6.0) / degree ** 1.5
        _run_steps(op, f, 12, dt)
        runs[guess] = (f.cpu().numpy(), op.diagnostics(f), op.cg_stats(), [t.cpu().numpy() for t in op.fields()])
    fp, dp, sp, (rp, pp, Ep) = runs["previous"]
    fl, dl, sl, (rl, pl, El) = runs["learned"]
    assert _rel(fl, fp) <= 1e-10
    assert _rel(El, Ep) <= 1e-8
    assert _rel(pl - pl.mean(), pp - pp.mean()) <= 1e-8
    assert abs(pl.mean()) <= 1e-12 * np.abs(pl).max()
    assert np.allclose(dl, dp, rtol=1e-8, atol=1e-14)
    assert sl["solves"] == sp["solves"] == 60
    assert sp["learned_picked"] == 0
    assert 0 < sl["learned_picked"] <= sl["solves"] - (1 if learn_fit == "least_squares" else 2)


def test_rhs_relative_tolerance():
    """cg_rhs_relative: the potential meets ||A phi - rhs|| <= tol ||rhs|| from any start."""
    dim_x, degree, cx, cv = 2, 3, 4, 6
    for guess in ("zero", "previous"):
        op, prob = _setup(dim_x, degree, cx, cv, guess=guess, cg_tol=1e-9, rhs_relative=True)
        f = op.initialize_dof_vector()
        op.interpolate(V.perturbed_maxwellian(dim_x, eps=0.05, perturbed_dims=(0, 1)), f)
        _run_steps(op, f, 2, 1e-3)
        op.solve_field(f)
        rho, phi, _ = (t.cpu().numpy() for t in op.fields())
        rhs = O.poisson_rhs(prob, rho)
        assert np.linalg.norm(O.poisson_apply(prob, phi) - rhs) <= 1.01e-9 * np.linalg.norm(rhs)
        st = op.cg_stats()
        assert st["solves"] == 11 and st["total_iterations"] >= st["last_iterations"]


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_fused_step_equals_unfused(dtype):
    """hd_vp_lsrk_step_fused (stage update inside the advection kernel, rotating vectors) against the
    reference's unfused stage sequence (hd_vp_lsrk_step)."""
    dim_x, degree, cx, cv = 2, 3, 4, 6
    out = {}
    for fused in (True, False):
        op, _ = _setup(dim_x, degree, cx, cv, dtype=dtype, guess="zero")
        f = op.initialize_dof_vector()
        op.interpolate(V.perturbed_maxwellian(dim_x, eps=0.05, perturbed_dims=(0, 1)), f)
        Ki, Ti = op.initialize_dof_vector(), op.initialize_dof_vector()
        integ = V.LowStorageRungeKuttaIntegrator(Ki, Ti, "rk45", fused=fused)
        for s in range(4):
            op.perform_time_step(integ, f, s * 1e-3, 1e-3)
        out[fused] = f.double().cpu().numpy()
    assert _rel(out[True], out[False]) <= (1e-12 if dtype == "f64" else 2e-6)


@pytest.mark.parametrize("dim_x,degree,cx,cv", CASES[:3])
def test_fp32x2_apply_matches_oracle(dim_x, degree, cx, cv):
    """FP64 storage with double-word FP32 advection contractions (hd_vp_set_arithmetic): the
    operator against the oracle at the FP64 bar of test_apply_matches_oracle, and against the
    native FP64 operator to 1e-12 (the field is solved identically in FP64 in both)."""
    op, prob = _setup(dim_x, degree, cx, cv)
    rng = np.random.default_rng(7 + dim_x * 10 + degree)
    fo = O.interpolate(prob, O.vp_initial_function(dim_x, dim_x, eps=0.2))
    fo = fo * (1.0 + 0.05 * rng.standard_normal(fo.size))
    src = torch.tensor(fo, device="cuda")
    nat = op.initialize_dof_vector()
    op.apply(nat, src, 0.0)
    op.set_arithmetic("fp32x2")
    x2 = op.initialize_dof_vector()
    op.apply(x2, src, 0.0)
    st = O.VPState(prob, 1e-12)
    ref = np.zeros_like(fo)
    st.operator(fo, ref, 0.0)
    assert _rel(x2.cpu().numpy(), ref) <= 1e-9
    assert _rel(x2.cpu().numpy(), nat.cpu().numpy()) <= 1e-12


def test_fp32x2_steps_equal_native():
    """Four fused rk45 steps of the 2x2v problem in FP32x2 and in native FP64 arithmetic: the
    distributions and the field energies agree to 1e-12; FP32 storage is refused."""
    dim_x, degree, cx, cv = 2, 3, 4, 6
    out, energy = {}, {}
    for ar in ("native", "fp32x2"):
        op, _ = _setup(dim_x, degree, cx, cv, guess="zero")
        op.set_arithmetic(ar)
        f = op.initialize_dof_vector()
        op.interpolate(V.perturbed_maxwellian(dim_x, eps=0.05, perturbed_dims=(0, 1)), f)
        _run_steps(op, f, 4, 1e-2)
        out[ar] = f.cpu().numpy()
        energy[ar] = op.diagnostics(f)
    assert _rel(out["fp32x2"], out["native"]) <= 1e-12
    assert _rel(energy["fp32x2"], energy["native"]) <= 1e-12
    op32, _ = _setup(dim_x, degree, cx, cv, dtype="f32")
    with pytest.raises(Exception):
        op32.set_arithmetic("fp32x2")


def _vp_benchmark_problem(guess, cells_v=32, learn_fit="least_squares"):
    """The 2x2v benchmark problem (16^2 x-cells, k = 3, rk45 at the benchmark's time step) with
    cells_v^2 v-cells, at a fixed CG accuracy ||r|| <= 1e-10 ||rhs||."""
    params = V.VlasovPoissonParameters(2, 3, [16, 16], [cells_v, cells_v], [0.0] * 2, [4 * math.pi] * 2,
                                       [-6.0] * 2, [6.0] * 2, dtype="f64", cg_tol=1e-10, guess=guess,
                                       cg_rhs_relative=True, learn_fit=learn_fit)
    op = V.VlasovPoissonOperation(params)
    f = op.initialize_dof_vector()
    op.interpolate(V.perturbed_maxwellian(2, eps=0.01, k=0.5, perturbed_dims=(0, 1)), f)
    Ki, Ti = op.initialize_dof_vector(), op.initialize_dof_vector()
    integ = V.LowStorageRungeKuttaIntegrator(Ki, Ti, "rk45")
    dt = V.time_step_rule(1.0, 0.05, min(4 * math.pi / 16, 12.0 / cells_v / 6.0), 3, 0.0, 1.0)
    return op, f, integ, dt


@pytest.mark.parametrize("learn_fit", ["least_squares", "adam"])
def test_learned_guess_saves_iterations(learn_fit):
    """What the trained network gains over the method without it, on the 2x2v benchmark problem
    (16^2 x-cells, 32^2 v-cells, k = 3): at a fixed accuracy (||r|| <= 1e-10 ||rhs||), once the
    model has seen a few solves, CG from the learned guess needs fewer iterations per solve than
    from the previous potential (the reference's start); the least-squares fit needs fewer than a
    quarter of those from either plain guess."""
    per_solve = {}
    for guess in ("previous", "zero", "learned"):
        op, f, integ, dt = _vp_benchmark_problem(guess, learn_fit=learn_fit)
        for s in range(3):
            op.perform_time_step(integ, f, s * dt, dt)
        st0 = op.cg_stats()
        for s in range(3, 13):
            op.perform_time_step(integ, f, s * dt, dt)
        st1 = op.cg_stats()
        per_solve[guess] = (st1["total_iterations"] - st0["total_iterations"]) / (st1["solves"] - st0["solves"])
        if guess == "learned":
            assert st1["learned_picked"] - st0["learned_picked"] > 0
    assert per_solve["learned"] < per_solve["previous"], per_solve
    if learn_fit == "least_squares":
        assert per_solve["learned"] < 0.25 * min(per_solve["previous"], per_solve["zero"]), per_solve


def test_learned_guess_faster_per_step():
    """The least-squares learned guess saves step time, not only iterations: FP64 rk45 steps of the
    2x2v problem (16^2 x-cells, 8^2 v-cells, so that the Poisson solve is a large share of a step)
    timed with CUDA events after warm-up steps are faster than from the zero guess and from the
    previous potential, the fields agreeing to the CG accuracy."""
    ms, energy = {}, {}
    for guess in ("previous", "zero", "learned"):
        op, f, integ, dt = _vp_benchmark_problem(guess, cells_v=8)
        t = 0.0
        for _ in range(4):
            op.perform_time_step(integ, f, t, dt)
            t += dt
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(20):
            op.perform_time_step(integ, f, t, dt)
            t += dt
        e1.record()
        torch.cuda.synchronize()
        ms[guess] = e0.elapsed_time(e1) / 20
        energy[guess] = op.diagnostics(f)[:2]
    assert ms["learned"] < 0.9 * min(ms["zero"], ms["previous"]), ms
    assert _rel(energy["learned"], energy["zero"]) <= 1e-8, energy


@pytest.mark.parametrize("dim_x,degree,cx,cv", [(1, 3, 8, 8), (2, 3, 4, 6), (2, 2, 3, 5), (3, 2, 2, 2)])
def test_block_jacobi_preconditioner_same_potential_fewer_iterations(dim_x, degree, cx, cv):
    """The cell-block Jacobi preconditioned CG (x-cell diagonal blocks of the SIPG matrix) meets the same
    accuracy, ||A phi - rhs|| <= tol ||rhs||, gives the same potential as unpreconditioned CG to that
    accuracy, and needs fewer iterations; degree 2 in 2D (9 DoFs per x-cell, not a divisor of the block
    size) takes the grid-barrier variant of the preconditioner step."""
    out = {}
    for pre in ("none", "block_jacobi"):
        op, prob = _setup(dim_x, degree, cx, cv, guess="zero", cg_tol=1e-11, rhs_relative=True, cg_precond=pre)
        f = op.initialize_dof_vector()
        op.interpolate(V.perturbed_maxwellian(dim_x, eps=0.05, perturbed_dims=tuple(range(dim_x))), f)
        # broadband noise in the density (as FP32 round-off brings in): many CG iterations without a preconditioner
        noise = np.random.default_rng(6).standard_normal(f.numel()) * 1e-3
        f += torch.tensor(noise, dtype=f.dtype, device="cuda")
        op.solve_field(f)
        rho, phi, _ = (t.cpu().numpy() for t in op.fields())
        rhs = O.poisson_rhs(prob, rho)
        assert np.linalg.norm(O.poisson_apply(prob, phi) - rhs) <= 1.01e-11 * np.linalg.norm(rhs)
        out[pre] = (phi - phi.mean(), op.cg_stats()["last_iterations"])
    assert _rel(out["block_jacobi"][0], out["none"][0]) <= 1e-8
    if dim_x == 1:  # on the 32-DoF 1D mesh the blocks remove at most an iteration or two
        assert out["block_jacobi"][1] <= out["none"][1], out
    else:
        assert out["block_jacobi"][1] < out["none"][1], out


@pytest.mark.parametrize("dim_x,degree,cx,cv,quadrature", [(1, 3, 8, 8, "gauss_lobatto"), (2, 3, 4, 4, "gauss_lobatto"),
                                                           (2, 2, 3, 5, "gauss_lobatto"), (2, 3, 4, 4, "gauss"),
                                                           (3, 2, 2, 2, "gauss_lobatto")])
def test_direct_poisson_solve_matches_cg(dim_x, degree, cx, cv, quadrature):
    """The direct solve (the SIPG matrix's pseudo-inverse, formed once by Gauss-Jordan elimination on the
    device) solves the oracle's system to round-off, gives the CG potential (CG to 1e-13) and field, the
    potential mean-free, with zero CG iterations counted per solve."""
    out = {}
    for solver in ("cg", "direct"):
        op, prob = _setup(dim_x, degree, cx, cv, guess="zero", cg_tol=1e-13, rhs_relative=True,
                          quadrature=quadrature, poisson_solver=solver)
        f = op.initialize_dof_vector()
        op.interpolate(V.perturbed_maxwellian(dim_x, eps=0.05, perturbed_dims=tuple(range(dim_x))), f)
        noise = np.random.default_rng(8).standard_normal(f.numel()) * 1e-3
        f += torch.tensor(noise, dtype=f.dtype, device="cuda")
        op.solve_field(f)
        rho, phi, E = (t.cpu().numpy() for t in op.fields())
        rhs = O.poisson_rhs(prob, rho)
        assert np.linalg.norm(O.poisson_apply(prob, phi) - rhs) <= 1e-11 * np.linalg.norm(rhs)
        st = op.cg_stats()
        out[solver] = (phi - phi.mean(), E, st)
    assert _rel(out["direct"][0], out["cg"][0]) <= 1e-10
    assert _rel(out["direct"][1], out["cg"][1]) <= 1e-10
    assert out["direct"][2]["solves"] == 1 and out["direct"][2]["last_iterations"] == 0
    assert out["cg"][2]["last_iterations"] > 0


def test_direct_poisson_solve_steps_and_limits():
    """Fused rk45 steps with the direct solve give the CG run's solution and field energy (CG to 1e-13;
    FP64 storage with native and FP32x2 advection, FP32 storage); x-spaces above 8192 DoFs are refused."""
    for dtype, tol in (("f64", 1e-12), ("f64x", 1e-12), ("f32", 2e-6)):
        res = {}
        for solver in ("cg", "direct"):
            op, _ = _setup(2, 3, 4, 4, dtype=dtype[:3], guess="zero", cg_tol=1e-13, rhs_relative=True,
                           poisson_solver=solver)
            if dtype == "f64x":
                op.set_arithmetic("fp32x2")
            f = op.initialize_dof_vector()
            op.interpolate(V.perturbed_maxwellian(2, eps=0.05, perturbed_dims=(0, 1)), f)
            hx, hv = 4 * math.pi / 4, 12.0 / 4
            _run_steps(op, f, 3, 0.05 * min(hx, hv / 6.0) / 3 ** 1.5)
            res[solver] = (f.double().cpu().numpy(), op.diagnostics(f))
        assert _rel(res["direct"][0], res["cg"][0]) <= tol
        assert _rel(res["direct"][1][:2], res["cg"][1][:2]) <= tol
    with pytest.raises(V.HdError):
        _setup(3, 3, 6, 2, poisson_solver="direct")  # 6^3 x-cells of 64 DoFs: 13,824 x-DoFs
