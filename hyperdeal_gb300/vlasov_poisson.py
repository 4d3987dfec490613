"""Host side of the Vlasov-Poisson right-hand side over the C ABI (hd_vp_*).

Mirrors the reference's Vlasov-Poisson example
(examples/vlasov_poisson/include/application.h:516-602): one operator
evaluation computes rho = int f dv, solves the SIPG Poisson problem for the
potential by conjugate gradients (FP64), takes grad(phi) at the x-nodes and
applies the upwind-DG advection with the phase-space velocity (v, grad phi).
The potential is kept between evaluations as the next CG initial guess (the
reference's behaviour); ``guess="learned"`` starts CG from a two-layer linear
network trained online on the solver's own (right-hand side, potential)
pairs: by default (``learn_fit="least_squares"``) the FP64 minimum-norm
least-squares fit of the recent pairs, computed inside the Poisson launch;
with ``learn_fit="adam"`` FP32 weights trained by Adam on the differences
between consecutive solves.  Diagnostics follow diagnostics.h:28-141.

Gauss-Lobatto collocation or Gauss quadrature, dim_x == dim_v, periodic x- and
v-meshes.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass
from typing import List, Sequence, Tuple

import torch

from . import _lib
from ._lib import HdError, check
from .advection import (Function, LowStorageRungeKuttaIntegrator, TimeLoop, _ptr, _stream, _swap_storage,
                        time_step_rule)

__all__ = ["VlasovPoissonParameters", "VlasovPoissonOperation", "perturbed_maxwellian", "run_hyperrectangle",
           "learn_loss_grad"]

_GUESS = {"zero": _lib.HD_VP_GUESS_ZERO, "previous": _lib.HD_VP_GUESS_PREVIOUS,
          "learned": _lib.HD_VP_GUESS_LEARNED}


@dataclass
class VlasovPoissonParameters:
    dim_x: int
    degree: int
    cells_x: Sequence[int]
    cells_v: Sequence[int]
    lo_x: Sequence[float]
    hi_x: Sequence[float]
    lo_v: Sequence[float]
    hi_v: Sequence[float]
    dtype: str = "f64"
    cg_tol: float = 1e-12
    cg_max_iter: int = 100000
    guess: str = "previous"
    learn_rank: int = 0
    learn_history: int = 0
    cg_rhs_relative: bool = False  # False: ||r|| <= cg_tol ||r_0|| as deal.II's ReductionControl
    learn_every: int = 0  # Adam steps every n-th solve (0: every solve)
    cg_precond: str = "block_jacobi"  # "none" or "block_jacobi" (x-cell diagonal blocks of the SIPG matrix)
    learn_fit: str = "least_squares"  # or "adam" (hd_vp_learn_fit)
    quadrature: str = "gauss_lobatto"  # or "gauss" (n_points = degree + 1, the reference's non-collocation runs)
    # "cg", or "direct": the SIPG matrix's pseudo-inverse kept in HBM, one matrix-vector product per solve
    # (x-spaces up to 8192 DoFs; guess and preconditioner unused)
    poisson_solver: str = "cg"

    def c(self) -> _lib.hd_vp_desc:
        d = _lib.hd_vp_desc()
        d.dim_x = d.dim_v = int(self.dim_x)
        d.degree = int(self.degree)
        d.dtype = _lib.HD_F64 if self.dtype == "f64" else _lib.HD_F32
        for i in range(self.dim_x):
            d.cells_x[i] = int(self.cells_x[i])
            d.cells_v[i] = int(self.cells_v[i])
            d.lo_x[i], d.hi_x[i] = float(self.lo_x[i]), float(self.hi_x[i])
            d.lo_v[i], d.hi_v[i] = float(self.lo_v[i]), float(self.hi_v[i])
        d.cg_tol = float(self.cg_tol)
        d.cg_max_iter = int(self.cg_max_iter)
        d.guess = _GUESS[self.guess]
        d.learn_rank = int(self.learn_rank)
        d.learn_history = int(self.learn_history)
        d.cg_rhs_relative = int(bool(self.cg_rhs_relative))
        d.learn_every = int(self.learn_every)
        d.cg_precond = {"none": _lib.HD_VP_PRECOND_NONE, "block_jacobi": _lib.HD_VP_PRECOND_BLOCK_JACOBI}[
            self.cg_precond]
        d.learn_fit = {"least_squares": _lib.HD_VP_FIT_LEAST_SQUARES, "adam": _lib.HD_VP_FIT_ADAM}[self.learn_fit]
        d.quadrature = {"gauss_lobatto": _lib.HD_QUAD_GAUSS_LOBATTO, "gauss": _lib.HD_QUAD_GAUSS}[self.quadrature]
        d.poisson_solver = {"cg": _lib.HD_VP_SOLVER_CG, "direct": _lib.HD_VP_SOLVER_DIRECT}[self.poisson_solver]
        return d


def perturbed_maxwellian(dim_x: int, eps: float = 0.01, k: float = 0.5, perturbed_dims: Sequence[int] = (0,)):
    """(1 + eps prod_{d in perturbed_dims} cos(k x_d)) prod_v exp(-v^2/2)/sqrt(2 pi)
    (examples/vlasov_poisson/cases/hyperrectangle.h:45-58 perturbs x_0)."""
    return Function(kind=3, amp=eps, omega=[k] * dim_x + [0.0] * dim_x,
                    cosine=[1 if d in perturbed_dims else 0 for d in range(dim_x)] + [2] * dim_x)


class VlasovPoissonOperation:
    """The Vlasov-Poisson right-hand side f -> -(v, grad phi[f]) . grad f in its DG form."""

    def __init__(self, params: VlasovPoissonParameters):
        self.params = params
        self._L = _lib.load()
        h = ctypes.c_void_p()
        desc = params.c()
        check(self._L.hd_vp_create(ctypes.byref(desc), ctypes.byref(h)))
        self._h = h
        self.n_dofs = int(self._L.hd_vp_n_dofs(h))
        self.n_dofs_x = int(self._L.hd_vp_n_dofs_x(h))
        self.dtype = torch.float64 if params.dtype == "f64" else torch.float32
        self.dim_x = params.dim_x

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.hd_vp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def initialize_dof_vector(self) -> torch.Tensor:
        return torch.zeros(self.n_dofs, dtype=self.dtype, device="cuda")

    def _check_vec(self, v: torch.Tensor, name: str) -> None:
        if not isinstance(v, torch.Tensor) or not v.is_cuda:
            raise HdError(_lib.HD_ERR_INVALID, "%s must be a CUDA tensor" % name)
        if v.dtype != self.dtype or v.numel() != self.n_dofs or not v.is_contiguous():
            raise HdError(_lib.HD_ERR_INVALID, "%s must be a contiguous %s vector of %d entries"
                          % (name, self.dtype, self.n_dofs))

    def interpolate(self, f: Function, dst: torch.Tensor, time: float = 0.0) -> None:
        self._check_vec(dst, "dst")
        fc = f.c()
        check(self._L.hd_vp_interpolate(self._h, ctypes.byref(fc), float(time), _ptr(dst), _stream()))

    def solve_field(self, f: torch.Tensor) -> None:
        self._check_vec(f, "f")
        check(self._L.hd_vp_solve_field(self._h, _ptr(f), _stream()))

    def apply(self, dst: torch.Tensor, src: torch.Tensor, time: float = 0.0) -> None:
        self._check_vec(dst, "dst")
        self._check_vec(src, "src")
        check(self._L.hd_vp_apply(self._h, _ptr(dst), _ptr(src), float(time), _stream()))

    # the LSRK operator signature op(src, dst, time)
    def __call__(self, src: torch.Tensor, dst: torch.Tensor, time: float) -> None:
        self.apply(dst, src, time)

    def perform_time_step(self, rk: LowStorageRungeKuttaIntegrator, solution: torch.Tensor, time: float,
                          dt: float) -> None:
        """One LSRK step with this operator entirely inside the library: the stage update fused
        into the advection kernel (hd_vp_lsrk_step_fused; the storages of solution and vec_Ki
        rotate as in LowStorageRungeKuttaIntegrator) unless the integrator was made with
        fused=False (hd_vp_lsrk_step: the reference's unfused stage sequence)."""
        for v, n in ((solution, "solution"), (rk.vec_Ki, "vec_Ki"), (rk.vec_Ti, "vec_Ti")):
            self._check_vec(v, n)
        if not rk.fused:
            check(self._L.hd_vp_lsrk_step(self._h, rk._h, _ptr(solution), _ptr(rk.vec_Ki), _ptr(rk.vec_Ti),
                                          float(time), float(dt), _stream()))
            return
        X = [ctypes.c_void_p(solution.data_ptr()), ctypes.c_void_p(rk.vec_Ki.data_ptr()),
             ctypes.c_void_p(rk.vec_Ti.data_ptr())]
        orig = [x.value for x in X]
        check(self._L.hd_vp_lsrk_step_fused(self._h, rk._h, ctypes.byref(X[0]), ctypes.byref(X[1]),
                                            ctypes.byref(X[2]), float(time), float(dt), _stream()))
        if X[0].value != orig[0]:
            assert X[0].value == orig[1] and X[1].value == orig[0]
            _swap_storage(solution, rk.vec_Ki)

    def fields(self) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
        """(rho, phi, E) of the last evaluation; E[(cell_x * n^dim_x + node) * dim_x + d] = d_d phi."""
        rho = torch.empty(self.n_dofs_x, dtype=torch.float64, device="cuda")
        phi = torch.empty_like(rho)
        E = torch.empty(self.n_dofs_x * self.dim_x, dtype=torch.float64, device="cuda")
        check(self._L.hd_vp_fields(self._h, _ptr(rho), _ptr(phi), _ptr(E), _stream()))
        return rho, phi, E

    def diagnostics(self, f: torch.Tensor) -> List[float]:
        """[field energy per x-direction, mass, L2 norm, kinetic energy, momentum per v-direction]."""
        self._check_vec(f, "f")
        n = self.dim_x + 3 + self.dim_x
        out = (ctypes.c_double * n)()
        check(self._L.hd_vp_diagnostics(self._h, _ptr(f), out, _stream()))
        return [float(out[i]) for i in range(n)]

    def cg_stats(self) -> dict:
        it = ctypes.c_int(0)
        tot = ctypes.c_longlong(0)
        solves = ctypes.c_longlong(0)
        res = ctypes.c_double(0.0)
        picked = ctypes.c_longlong(0)
        check(self._L.hd_vp_cg_stats(self._h, ctypes.byref(it), ctypes.byref(tot), ctypes.byref(solves),
                                     ctypes.byref(res), ctypes.byref(picked)))
        return {"last_iterations": it.value, "total_iterations": tot.value, "solves": solves.value,
                "last_residual": res.value, "learned_picked": picked.value}

    def set_arithmetic(self, arithmetic: str) -> None:
        """'native' (FP64 advection contractions) or 'fp32x2' (double-word FP32
        contractions on FP64 storage; the Poisson solve stays FP64)."""
        v = {"native": _lib.HD_ARITH_NATIVE, "fp32x2": _lib.HD_ARITH_FP32X2}[arithmetic]
        check(self._L.hd_vp_set_arithmetic(self._h, v))

    def set_guess(self, guess: str) -> None:
        check(self._L.hd_vp_set_guess(self._h, _GUESS[guess]))

    def set_kernel(self, kernel: str) -> None:
        """FP32 advection kernel: 'auto' (the TMA-pipelined kernel where it applies), 'generic' or
        'pipelined' (hd_vp_set_kernel)."""
        v = {"auto": _lib.HD_KERNEL_AUTO, "generic": _lib.HD_KERNEL_GENERIC,
             "pipelined": _lib.HD_KERNEL_PIPELINED}[kernel]
        check(self._L.hd_vp_set_kernel(self._h, v))

    @property
    def kernel(self) -> str:
        return {_lib.HD_KERNEL_GENERIC: "generic", _lib.HD_KERNEL_PIPELINED: "pipelined"}[
            self._L.hd_vp_kernel(self._h)]

    def device_status(self) -> int:
        """Status of the pipelined advection since the last call (synchronises, resets it)."""
        st = ctypes.c_int(0)
        check(self._L.hd_vp_device_status(self._h, ctypes.byref(st)))
        return st.value

    def set_wait_test(self, wait_limit: int, skip_issue: int) -> None:
        check(self._L.hd_vp_set_wait_test(self._h, wait_limit, skip_issue))


def learn_loss_grad(W1: torch.Tensor, W2: torch.Tensor, X: torch.Tensor, Y: torch.Tensor):
    """loss = 1/(2B) sum_b ||W2 W1 x_b - y_b||^2 and (dW1, dW2) from the learned guess's own
    training kernels.  W1: r x n, W2: n x r, X, Y: B x n (float32, CUDA, contiguous)."""
    L = _lib.load()
    r, n = W1.shape
    B = X.shape[0]
    for t in (W1, W2, X, Y):
        if t.dtype != torch.float32 or not t.is_cuda or not t.is_contiguous():
            raise HdError(_lib.HD_ERR_INVALID, "learn_loss_grad wants contiguous float32 CUDA tensors")
    if W2.shape != (n, r) or X.shape != (B, n) or Y.shape != (B, n):
        raise HdError(_lib.HD_ERR_INVALID, "learn_loss_grad: shape mismatch")
    dW1 = torch.empty_like(W1)
    dW2 = torch.empty_like(W2)
    loss = torch.empty(1, dtype=torch.float32, device=W1.device)
    check(L.hd_vp_learn_loss_grad(n, r, B, _ptr(W1), _ptr(W2), _ptr(X), _ptr(Y), _ptr(dW1), _ptr(dW2),
                                  _ptr(loss), _stream()))
    return float(loss.item()), dW1, dW2


def run_hyperrectangle(dim_x: int = 2, degree: int = 3, cells_x: int = 4, cells_v: int = 4, dtype: str = "f64",
                       final_time: float = 0.5, time_step: float = 0.1, cfl: float = 0.05, tick: float = 0.1,
                       rk: str = "rk45", cg_tol: float = 1e-12, guess: str = "previous",
                       quadrature: str = "gauss_lobatto", poisson_solver: str = "cg"):
    """The reference's Vlasov-Poisson application on its hyperrectangle case: x in [0, 4 pi]^dim_x,
    v in [-6, 6]^dim_x, periodic, the time-step rule with transport velocity (1, .., 6, ..)
    (examples/vlasov_poisson/cases/hyperrectangle.h, application.h:345-602).  Returns the
    diagnostics rows (time, field energy per x-direction, mass, L2, kinetic energy, momentum)
    and the operator."""
    params = VlasovPoissonParameters(dim_x, degree, [cells_x] * dim_x, [cells_v] * dim_x, [0.0] * dim_x,
                                     [4 * math.pi] * dim_x, [-6.0] * dim_x, [6.0] * dim_x, dtype=dtype,
                                     cg_tol=cg_tol, guess=guess, quadrature=quadrature,
                                     poisson_solver=poisson_solver)
    op = VlasovPoissonOperation(params)
    sol = op.initialize_dof_vector()
    op.interpolate(perturbed_maxwellian(dim_x), sol)
    # cfl.h:56-124 with the constant transport velocity of the case
    hx = 4 * math.pi / cells_x
    hv = 12.0 / cells_v
    critical = min(1.0 / (1.0 / hx), 1.0 / (6.0 / hv))
    dt = time_step_rule(time_step, cfl, critical, degree, 0.0, final_time)
    Ki = op.initialize_dof_vector()
    Ti = op.initialize_dof_vector()
    integ = LowStorageRungeKuttaIntegrator(Ki, Ti, rk)
    rows = []

    def step(u, t, h, _op):
        op.perform_time_step(integ, u, t, h)

    def diag(t):
        # output when a multiple of `tick` was crossed in the last step
        # (examples/vlasov_poisson/include/application.h, as the advection example's :464-471)
        if t == 0.0 or int((t + 1e-11) / tick) != int((t + 1e-11 - dt) / tick):
            rows.append((t,) + tuple(op.diagnostics(sol)))

    TimeLoop(dt, 0.0, final_time).loop(sol, step, op, diag)
    return rows, op
