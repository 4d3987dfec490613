"""Host-side mirror of hyper.deal's advection interface over the C ABI.

Names, argument meaning and error behaviour follow the reference:

* ``AdvectionOperation.apply(dst, src, time)`` --
  include/hyper.deal/operators/advection/advection_operation.h:134-209
  (dst is overwritten, ECL branch).
* ``LowStorageRungeKuttaIntegrator(vec_Ki, vec_Ti, type, only_Ti_is_ghosted)``
  with ``perform_time_step(solution, current_time, time_step, op)`` and
  ``n_stages()`` -- include/hyper.deal/base/time_integrators.h:47-115.
* ``TimeLoop.loop`` -- source/base/time_loop.cc:33-67.
* ``VectorTools.interpolate`` / ``norm_and_error`` --
  include/hyper.deal/numerics/vector_tools.h:81-223.
* ``compute_critical_time_step`` -- operators/advection/cfl.h:56-124.

Vectors are CUDA tensors (torch provides device memory and streams); all work
runs in the CUDA library through include/hyperdeal_gb300.h.  Errors raise
``HdError`` (the reference throws ``dealii::ExceptionBase``).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field
from typing import Callable, Optional, Sequence

import torch

from . import _lib
from ._lib import HdError, check

__all__ = ["Function", "AdvectionParameters", "AdvectionOperation", "LowStorageRungeKuttaIntegrator",
           "TimeLoop", "VectorTools", "compute_critical_time_step", "time_step_rule", "HdError"]


@dataclass
class Function:
    """amp * prod_d trig_d(omega_d (x_d - speed_d t) + phase_d) (kind 2), a constant (kind 1) or 0."""
    kind: int = 2
    amp: float = 1.0
    omega: Sequence[float] = ()
    speed: Sequence[float] = ()
    phase: Sequence[float] = ()
    cosine: Sequence[int] = ()

    def c(self) -> _lib.hd_function:
        f = _lib.hd_function()
        f.kind = int(self.kind)
        f.amp = float(self.amp)
        for name in ("omega", "speed", "phase"):
            arr = getattr(f, name)
            for i, v in enumerate(getattr(self, name)):
                arr[i] = float(v)
        for i, v in enumerate(self.cosine):
            f.cosine[i] = int(v)
        return f


@dataclass
class AdvectionParameters:
    """Everything the reference's MatrixFree + AdvectionOperation::reinit receive for a
    Cartesian phase-space mesh (NRefinements = 0)."""
    dim_x: int
    dim_v: int
    degree: int
    cells_x: Sequence[int]
    cells_v: Sequence[int]
    lo_x: Sequence[float]
    hi_x: Sequence[float]
    lo_v: Sequence[float]
    hi_v: Sequence[float]
    velocity: Sequence[float]
    periodic_x: bool = True
    periodic_v: bool = True
    skew: float = 0.0
    dtype: str = "f64"
    boundary: Optional[Function] = None  # None: homogeneous Dirichlet on non-periodic faces
    quadrature: str = "gauss_lobatto"  # "gauss_lobatto" (collocation) or "gauss"

    def c(self) -> _lib.hd_adv_desc:
        d = _lib.hd_adv_desc()
        d.dim_x, d.dim_v, d.degree = self.dim_x, self.dim_v, self.degree
        d.n_points = self.degree + 1
        d.dtype = {"f64": _lib.HD_F64, "f32": _lib.HD_F32}[self.dtype]
        for i in range(self.dim_x):
            d.cells_x[i] = int(self.cells_x[i])
            d.lo_x[i] = float(self.lo_x[i])
            d.hi_x[i] = float(self.hi_x[i])
        for i in range(self.dim_v):
            d.cells_v[i] = int(self.cells_v[i])
            d.lo_v[i] = float(self.lo_v[i])
            d.hi_v[i] = float(self.hi_v[i])
        d.periodic_x, d.periodic_v = int(self.periodic_x), int(self.periodic_v)
        for i, v in enumerate(self.velocity):
            d.velocity[i] = float(v)
        d.skew = float(self.skew)
        if self.boundary is not None:
            d.bc_kind = _lib.HD_BC_FUNCTION
            d.bc = self.boundary.c()
        d.quadrature = {"gauss_lobatto": _lib.HD_QUAD_GAUSS_LOBATTO, "gauss": _lib.HD_QUAD_GAUSS}[self.quadrature]
        return d


def _stream() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t: torch.Tensor) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


class AdvectionOperation:
    """Upwind-DG advection operator on the phase space (ECL, Gauss-Lobatto collocation)."""

    def __init__(self, params: AdvectionParameters):
        self.params = params
        self._L = _lib.load()
        h = ctypes.c_void_p()
        desc = params.c()
        check(self._L.hd_adv_create(ctypes.byref(desc), ctypes.byref(h)))
        self._h = h
        self.n_dofs = int(self._L.hd_adv_n_dofs(h))
        self.dtype = torch.float64 if params.dtype == "f64" else torch.float32
        self.dim = params.dim_x + params.dim_v

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.hd_adv_destroy(self._h)
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

    def apply(self, dst: torch.Tensor, src: torch.Tensor, time: float = 0.0) -> None:
        self._check_vec(dst, "dst")
        self._check_vec(src, "src")
        check(self._L.hd_adv_apply(self._h, _ptr(dst), _ptr(src), float(time), _stream()))

    # the LSRK operator signature op(src, dst, time) of the reference's lambdas
    def __call__(self, src: torch.Tensor, dst: torch.Tensor, time: float) -> None:
        self.apply(dst, src, time)

    def critical_time_step(self) -> float:
        return float(self._L.hd_adv_critical_time_step(self._h))

    def set_kernel(self, variant: str) -> None:
        """'auto', 'generic' or 'pipelined' (see hd_adv_set_kernel)."""
        v = {"auto": _lib.HD_KERNEL_AUTO, "generic": _lib.HD_KERNEL_GENERIC,
             "pipelined": _lib.HD_KERNEL_PIPELINED}[variant]
        check(self._L.hd_adv_set_kernel(self._h, v))

    @property
    def kernel(self) -> str:
        return {_lib.HD_KERNEL_GENERIC: "generic", _lib.HD_KERNEL_PIPELINED: "pipelined"}[
            int(self._L.hd_adv_kernel(self._h))]

    def set_arithmetic(self, arithmetic: str) -> None:
        """'native' (FP64 contractions) or 'fp32x2' (double-word FP32 contractions
        on FP64 storage; see hd_adv_set_arithmetic)."""
        v = {"native": _lib.HD_ARITH_NATIVE, "fp32x2": _lib.HD_ARITH_FP32X2}[arithmetic]
        check(self._L.hd_adv_set_arithmetic(self._h, v))

    @property
    def arithmetic(self) -> str:
        return {_lib.HD_ARITH_NATIVE: "native", _lib.HD_ARITH_FP32X2: "fp32x2"}[
            int(self._L.hd_adv_arithmetic(self._h))]

    def set_tile(self, cells_per_cta: int = 0, ctas_per_sm: int = 0) -> None:
        """Tile of the generic kernel (hd_adv_set_tile); 0 = default."""
        check(self._L.hd_adv_set_tile(self._h, int(cells_per_cta), int(ctas_per_sm)))

    def autotune(self, src: torch.Tensor, dst: torch.Tensor, reps: int = 3) -> dict:
        """Time candidate tiles with apply launches (src read, dst overwritten) and keep the fastest."""
        self._check_vec(src, "src")
        self._check_vec(dst, "dst")
        c, p, ms = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_double(0.0)
        check(self._L.hd_adv_autotune(self._h, _ptr(src), _ptr(dst), int(reps), ctypes.byref(c), ctypes.byref(p),
                                      ctypes.byref(ms), _stream()))
        return {"cells_per_cta": c.value, "ctas_per_sm": p.value, "ms_per_apply": ms.value}

    def tile_limits(self):
        """(max cells per CTA, threads per cell) of the generic kernel for this operator."""
        a, b = ctypes.c_int(0), ctypes.c_int(0)
        check(self._L.hd_adv_tile_limits(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def set_wait_test(self, wait_limit: int = 0, skip_issue: int = -1) -> None:
        """Test hook of the pipelined kernel's bounded waits (hd_adv_set_wait_test)."""
        check(self._L.hd_adv_set_wait_test(self._h, int(wait_limit), int(skip_issue)))

    def device_status(self) -> int:
        """Error code recorded by the device since the last call (0 = none); synchronises."""
        st = ctypes.c_int(0)
        check(self._L.hd_adv_device_status(self._h, ctypes.byref(st)))
        return int(st.value)


def compute_critical_time_step(op: AdvectionOperation) -> float:
    return op.critical_time_step()


def time_step_rule(time_step: float, cfl: float, critical: float, degree: int, start: float, final: float) -> float:
    """examples/advection/include/application.h:377-392"""
    dt = min(time_step, cfl * critical / degree ** 1.5)
    return (final - start) / math.ceil((final - start) / dt)


def _swap_storage(a: torch.Tensor, b: torch.Tensor) -> None:
    tmp = a.data
    a.data = b.data
    b.data = tmp


class LowStorageRungeKuttaIntegrator:
    """Kennedy-Carpenter-Lewis low-storage explicit RK (rk33, rk45, rk47, rk59).

    ``perform_time_step(solution, t, dt, op)``: when ``op`` is an AdvectionOperation the
    stage operator and the vector update run fused in one kernel per stage; the three
    vectors then rotate roles and their storages are swapped back so that ``solution``
    holds the new state (``vec_Ki``/``vec_Ti`` are scratch, as in the reference).  Any
    other callable ``op(src, dst, t)`` runs the reference's unfused sequence.
    """

    def __init__(self, vec_Ki: torch.Tensor, vec_Ti: torch.Tensor, type: str = "rk45",
                 only_Ti_is_ghosted: bool = True, fused: bool = True):
        self._L = _lib.load()
        h = ctypes.c_void_p()
        check(self._L.hd_lsrk_create(type.encode(), ctypes.byref(h)))
        self._h = h
        self.vec_Ki = vec_Ki
        self.vec_Ti = vec_Ti
        self.type = type
        self.only_Ti_is_ghosted = only_Ti_is_ghosted
        self.fused = fused
        ns = self.n_stages()
        ai = (ctypes.c_double * 16)()
        bi = (ctypes.c_double * 16)()
        ci = (ctypes.c_double * 16)()
        check(self._L.hd_lsrk_coefficients(h, ai, bi, ci))
        self.ai = [ai[i] for i in range(ns - 1)]
        self.bi = [bi[i] for i in range(ns)]
        self.ci = [ci[i] for i in range(ns)]

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.hd_lsrk_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def n_stages(self) -> int:
        return int(self._L.hd_lsrk_n_stages(self._h))

    def perform_time_step(self, solution: torch.Tensor, current_time: float, time_step: float,
                          op: Callable) -> None:
        if isinstance(op, AdvectionOperation):
            for v, n in ((solution, "solution"), (self.vec_Ki, "vec_Ki"), (self.vec_Ti, "vec_Ti")):
                op._check_vec(v, n)
            if self.fused:
                X = [ctypes.c_void_p(solution.data_ptr()), ctypes.c_void_p(self.vec_Ki.data_ptr()),
                     ctypes.c_void_p(self.vec_Ti.data_ptr())]
                orig = [x.value for x in X]
                check(self._L.hd_lsrk_step(op.handle, self._h, ctypes.byref(X[0]), ctypes.byref(X[1]),
                                           ctypes.byref(X[2]), float(current_time), float(time_step), _stream()))
                # the new solution lives in the storage that was vec_Ki; rotate storages
                if X[0].value != orig[0]:
                    assert X[0].value == orig[1] and X[1].value == orig[0]
                    _swap_storage(solution, self.vec_Ki)
                return
            check(self._L.hd_lsrk_step_unfused(op.handle, self._h, _ptr(solution), _ptr(self.vec_Ki),
                                               _ptr(self.vec_Ti), float(current_time), float(time_step),
                                               _stream()))
            return
        # generic operator: the reference's stage sequence with the CUDA vector update
        dtype = _lib.HD_F64 if solution.dtype == torch.float64 else _lib.HD_F32
        n = solution.numel()
        if self.only_Ti_is_ghosted:
            self.vec_Ti.copy_(solution)
            cur = self.vec_Ti
        else:
            cur = solution
        ns = self.n_stages()
        for s in range(ns):
            op(cur, self.vec_Ki, current_time + self.ci[s] * time_step)
            ai = 0.0 if s == ns - 1 else self.ai[s] * time_step
            check(self._L.hd_lsrk_stage_update(dtype, n, self.bi[s] * time_step, ai, _ptr(self.vec_Ki),
                                               _ptr(solution), _ptr(self.vec_Ti), _stream()))
            cur = self.vec_Ti


class TimeLoop:
    """source/base/time_loop.cc:33-67"""

    def __init__(self, time_step: float, start_time: float, final_time: float, max_time_step_number: int = 100000000):
        self.time_step = time_step
        self.start_time = start_time
        self.final_time = final_time
        self.max_time_step_number = max_time_step_number

    def loop(self, solution, time_integrator: Callable, runnable: Callable, diagnostics: Callable) -> int:
        n = 1
        diagnostics(self.start_time)
        t = self.start_time + self.time_step
        while t <= self.final_time * 1.0000000000001 and n <= self.max_time_step_number:
            time_integrator(solution, t - self.time_step, self.time_step, runnable)
            diagnostics(t)
            t += self.time_step
            n += 1
        return n - 1


class VectorTools:
    @staticmethod
    def interpolate(op: AdvectionOperation, f: Function, dst: torch.Tensor, time: float = 0.0) -> None:
        op._check_vec(dst, "dst")
        fc = f.c()
        check(op._L.hd_interpolate(op.handle, ctypes.byref(fc), float(time), _ptr(dst), _stream()))

    @staticmethod
    def norm_and_error(op: AdvectionOperation, f: Function, src: torch.Tensor, time: float = 0.0):
        op._check_vec(src, "src")
        fc = f.c()
        out = (ctypes.c_double * 2)()
        check(op._L.hd_norm_and_error(op.handle, ctypes.byref(fc), float(time), _ptr(src), out, _stream()))
        return float(out[0]), float(out[1])
