"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle restates hyper.deal's phase-space advection path on the CPU
(hd_oracle.c).  Only the test suite, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module: it is the checker for the
CUDA path, never the thing measured or shipped.

Besides the C entry points it restates the advection application's driver
logic used by the reference's golden tests:

* time-step rule: examples/advection/include/application.h:363-396
* time loop and diagnostics tick: source/base/time_loop.cc:33-67 and
  examples/advection/include/application.h:464-506
* ``hyperrectangle`` case (exact solution, domain [-1,1]^D, Dirichlet data):
  examples/advection/cases/hyperrectangle.h:29-66, :220-235
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libhd_oracle.so")
MAX_DIM = 6


def build(force: bool = False) -> str:
    """Compile hd_oracle.c into oracle/_build/libhd_oracle.so (gcc, OpenMP)."""
    src = os.path.join(HERE, "hd_oracle.c")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(os.path.join(HERE, "hd_oracle.h"))):
        return LIB_PATH
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11",
                           "-D_DEFAULT_SOURCE", "-o", tmp, src, "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class Func(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("amp", ctypes.c_double),
                ("omega", ctypes.c_double * MAX_DIM), ("speed", ctypes.c_double * MAX_DIM),
                ("phase", ctypes.c_double * MAX_DIM), ("cosine", ctypes.c_int * MAX_DIM)]


class _Problem(ctypes.Structure):
    _fields_ = [("dim_x", ctypes.c_int), ("dim_v", ctypes.c_int), ("degree", ctypes.c_int),
                ("n_points", ctypes.c_int), ("collocation", ctypes.c_int),
                ("cells", ctypes.c_int * MAX_DIM), ("lo", ctypes.c_double * MAX_DIM),
                ("hi", ctypes.c_double * MAX_DIM), ("periodic_x", ctypes.c_int),
                ("periodic_v", ctypes.c_int), ("velocity", ctypes.c_double * MAX_DIM),
                ("skew", ctypes.c_double), ("bc_inhomogeneous", ctypes.c_int),
                ("bc_func", Func), ("n_threads", ctypes.c_int), ("efield", ctypes.POINTER(ctypes.c_double))]


def make_func(kind: int = 2, amp: float = 1.0, omega: Sequence[float] = (), speed: Sequence[float] = (),
              phase: Sequence[float] = (), cosine: Sequence[int] = ()) -> Func:
    f = Func()
    f.kind = kind
    f.amp = amp
    for i, v in enumerate(omega):
        f.omega[i] = v
    for i, v in enumerate(speed):
        f.speed[i] = v
    for i, v in enumerate(phase):
        f.phase[i] = v
    for i, v in enumerate(cosine):
        f.cosine[i] = int(v)
    return f


def eval_func(f: Func, x: np.ndarray, t: float) -> np.ndarray:
    """numpy evaluation of an hdo_func at points x[..., D]."""
    D = x.shape[-1]
    if f.kind == 0:
        return np.zeros(x.shape[:-1])
    if f.kind == 1:
        return np.full(x.shape[:-1], f.amp)
    r = np.full(x.shape[:-1], f.amp)
    for d in range(D):
        arg = f.omega[d] * (x[..., d] - f.speed[d] * t) + f.phase[d]
        r = r * (np.cos(arg) if f.cosine[d] else np.sin(arg))
    return r


@dataclass
class Problem:
    dim_x: int
    dim_v: int
    degree: int
    cells: Sequence[int]
    lo: Sequence[float]
    hi: Sequence[float]
    velocity: Sequence[float]
    periodic_x: bool = True
    periodic_v: bool = True
    collocation: bool = True
    skew: float = 0.0
    bc_func: Optional[Func] = None
    n_threads: int = 0

    @property
    def dim(self) -> int:
        return self.dim_x + self.dim_v

    @property
    def n_dofs(self) -> int:
        return int(np.prod(self.cells)) * (self.degree + 1) ** self.dim

    def c(self) -> _Problem:
        p = _Problem()
        p.dim_x, p.dim_v, p.degree = self.dim_x, self.dim_v, self.degree
        p.n_points = self.degree + 1
        p.collocation = int(self.collocation)
        for d in range(self.dim):
            p.cells[d] = int(self.cells[d])
            p.lo[d] = float(self.lo[d])
            p.hi[d] = float(self.hi[d])
            p.velocity[d] = float(self.velocity[d])
        p.periodic_x, p.periodic_v = int(self.periodic_x), int(self.periodic_v)
        p.skew = float(self.skew)
        if self.bc_func is not None:
            p.bc_inhomogeneous = 1
            p.bc_func = self.bc_func
        p.n_threads = int(self.n_threads)
        return p


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        P = ctypes.POINTER(_Problem)
        L.hdo_apply.argtypes = [P, dp, dp, ctypes.c_double]
        L.hdo_apply_cells.argtypes = [P, dp, dp, ctypes.c_double, ctypes.POINTER(ctypes.c_longlong),
                                      ctypes.c_longlong]
        L.hdo_apply_cells_f32.argtypes = [P, ctypes.POINTER(ctypes.c_float), dp, ctypes.c_double,
                                          ctypes.POINTER(ctypes.c_longlong), ctypes.c_longlong]
        L.hdo_lsrk_step.argtypes = [P, ctypes.c_char_p, dp, dp, dp, ctypes.c_double, ctypes.c_double]
        L.hdo_interpolate.argtypes = [P, ctypes.POINTER(Func), ctypes.c_double, dp]
        L.hdo_norm_and_error.argtypes = [P, ctypes.POINTER(Func), ctypes.c_double, dp, dp]
        L.hdo_critical_time_step.argtypes = [P]
        L.hdo_critical_time_step.restype = ctypes.c_double
        L.hdo_gauss_lobatto.argtypes = [ctypes.c_int, dp, dp]
        L.hdo_gauss.argtypes = [ctypes.c_int, dp, dp]
        L.hdo_lsrk_coefficients.argtypes = [ctypes.c_char_p, dp, dp]
        L.hdo_velocity_moment.argtypes = [P, dp, dp]
        L.hdo_coordinate_moment.argtypes = [P, dp, dp]
        L.hdo_n_dofs.argtypes = [P]
        L.hdo_n_dofs.restype = ctypes.c_longlong
        L.hdo_poisson_apply.argtypes = [P, dp, dp]
        L.hdo_poisson_rhs.argtypes = [P, dp, dp]
        L.hdo_poisson_solve.argtypes = [P, dp, dp, ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        L.hdo_vp_field.argtypes = [P, dp, dp]
        L.hdo_vp_operator.argtypes = [P, dp, dp, ctypes.c_double, dp, dp, ctypes.c_double,
                                      ctypes.POINTER(ctypes.c_int)]
        L.hdo_vp_diagnostics.argtypes = [P, dp, dp, dp]
        OPF = ctypes.CFUNCTYPE(None, dp, dp, ctypes.c_double, ctypes.c_void_p)
        L.hdo_lsrk_step_op.argtypes = [ctypes.c_longlong, ctypes.c_char_p, dp, dp, dp,
                                       ctypes.c_double, ctypes.c_double, OPF, ctypes.c_void_p]
        L._OPF = OPF
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _check(rc: int, what: str):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed ({rc})")


def apply(p: Problem, src: np.ndarray, time: float = 0.0) -> np.ndarray:
    dst = np.empty_like(src)
    cp = p.c()
    _check(lib().hdo_apply(ctypes.byref(cp), _ptr(src), _ptr(dst), time), "apply")
    return dst


def apply_cells(p: Problem, src: np.ndarray, cells, time: float = 0.0) -> np.ndarray:
    """Operator values at the listed cells only: [len(cells), (k+1)^D] in float64.
    ``src`` may be float64 or float32 (widened to double on read)."""
    cells = np.ascontiguousarray(cells, dtype=np.int64)
    nc = (p.degree + 1) ** p.dim
    dst = np.zeros((cells.size, nc))
    cp = p.c()
    cptr = cells.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))
    if src.dtype == np.float32:
        assert src.flags.c_contiguous
        rc = lib().hdo_apply_cells_f32(ctypes.byref(cp), src.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                       _ptr(dst), time, cptr, cells.size)
    else:
        rc = lib().hdo_apply_cells(ctypes.byref(cp), _ptr(src), _ptr(dst), time, cptr, cells.size)
    _check(rc, "apply_cells")
    return dst


def lsrk_step(p: Problem, rk: str, sol: np.ndarray, time: float, dt: float,
              Ki: Optional[np.ndarray] = None, Ti: Optional[np.ndarray] = None) -> None:
    Ki = np.empty_like(sol) if Ki is None else Ki
    Ti = np.empty_like(sol) if Ti is None else Ti
    cp = p.c()
    _check(lib().hdo_lsrk_step(ctypes.byref(cp), rk.encode(), _ptr(sol), _ptr(Ki), _ptr(Ti), time, dt),
           "lsrk_step")


def lsrk_step_op(rk: str, sol: np.ndarray, time: float, dt: float,
                 op: Callable[[np.ndarray, np.ndarray, float], None]) -> None:
    n = sol.size
    Ki = np.zeros_like(sol)
    Ti = np.zeros_like(sol)
    L = lib()

    def cb(src, dst, t, _ctx):
        s = np.ctypeslib.as_array(src, shape=(n,))
        d = np.ctypeslib.as_array(dst, shape=(n,))
        op(s, d, t)

    f = L._OPF(cb)
    _check(L.hdo_lsrk_step_op(n, rk.encode(), _ptr(sol), _ptr(Ki), _ptr(Ti), time, dt, f, None), "lsrk_step_op")


def lsrk_coefficients(rk: str):
    a = np.zeros(16)
    b = np.zeros(16)
    ns = lib().hdo_lsrk_coefficients(rk.encode(), _ptr(a), _ptr(b))
    if ns == 0:
        raise ValueError(rk)
    return a[:ns - 1].copy(), b[:ns].copy()


def interpolate(p: Problem, f: Func, time: float = 0.0) -> np.ndarray:
    dst = np.empty(p.n_dofs)
    cp = p.c()
    _check(lib().hdo_interpolate(ctypes.byref(cp), ctypes.byref(f), time, _ptr(dst)), "interpolate")
    return dst


def norm_and_error(p: Problem, f: Func, time: float, src: np.ndarray):
    out = np.zeros(2)
    cp = p.c()
    _check(lib().hdo_norm_and_error(ctypes.byref(cp), ctypes.byref(f), time, _ptr(src), _ptr(out)),
           "norm_and_error")
    return float(out[0]), float(out[1])


def critical_time_step(p: Problem) -> float:
    cp = p.c()
    return lib().hdo_critical_time_step(ctypes.byref(cp))


def velocity_moment(p: Problem, src: np.ndarray) -> np.ndarray:
    nx = int(np.prod(p.cells[:p.dim_x])) * (p.degree + 1) ** p.dim_x
    rho = np.zeros(nx)
    cp = p.c()
    _check(lib().hdo_velocity_moment(ctypes.byref(cp), _ptr(src), _ptr(rho)), "velocity_moment")
    return rho


def coordinate_moment(p: Problem, src: np.ndarray) -> np.ndarray:
    """The integral over x of f at every v-DoF (vector_tools.h:317-400)."""
    nv = int(np.prod(p.cells[p.dim_x:])) * (p.degree + 1) ** p.dim_v
    out = np.zeros(nv)
    cp = p.c()
    _check(lib().hdo_coordinate_moment(ctypes.byref(cp), _ptr(src), _ptr(out)), "coordinate_moment")
    return out


def node_coordinates(p: Problem) -> np.ndarray:
    """Coordinates (n_dofs x dim) of the Gauss-Lobatto support points in the DoF order: cell gid =
    gid_x + n_cells_x gid_v with lexicographic x- and v-cells, nodes lexicographic inside a cell
    (matrix_free.templates.h:535-563, shape_info.h:141-160)."""
    n = p.degree + 1
    D = p.dim
    xi, _ = gauss_lobatto(n)
    cells = [int(c) for c in p.cells]
    h = [(p.hi[d] - p.lo[d]) / cells[d] for d in range(D)]
    # cell coordinates: x-cells (first direction fastest), then v-cells
    cell_axes = np.meshgrid(*[np.arange(c) for c in reversed(cells)], indexing="ij")
    cc = [a.reshape(-1) for a in reversed(cell_axes)]  # cc[d][gid]
    node_axes = np.meshgrid(*[np.arange(n)] * D, indexing="ij")
    nn = [a.reshape(-1) for a in reversed(node_axes)]  # nn[d][node]
    out = np.empty((len(cc[0]) * n ** D, D))
    for d in range(D):
        out[:, d] = (p.lo[d] + (cc[d][:, None] + xi[nn[d]][None, :]) * h[d]).reshape(-1)
    return out


def gauss_lobatto(n: int):
    x = np.zeros(n)
    w = np.zeros(n)
    _check(lib().hdo_gauss_lobatto(n, _ptr(x), _ptr(w)), "gauss_lobatto")
    return x, w


def gauss(n: int):
    x = np.zeros(n)
    w = np.zeros(n)
    _check(lib().hdo_gauss(n, _ptr(x), _ptr(w)), "gauss")
    return x, w


# --------------------------------------------------------------------------
# driver logic of the reference's advection application
# --------------------------------------------------------------------------

def time_step_rule(time_step: float, cfl: float, critical: float, degree: int,
                   start: float, final: float) -> float:
    """dt = min(TimeStep, CFL * dt_crit / k^1.5), then T / ceil(T / dt)
    (examples/advection/include/application.h:363-396)."""
    dt = min(time_step, cfl * critical / degree ** 1.5)
    return (final - start) / math.ceil((final - start) / dt)


def time_loop(start: float, final: float, dt: float, step: Callable[[float, float], None],
              diagnostics: Callable[[float], None], max_steps: int = 100000000) -> int:
    """source/base/time_loop.cc:33-67 (final_time * (1 + 1e-13) guard)."""
    n = 1
    diagnostics(start)
    t = start + dt
    while t <= final * 1.0000000000001 and n <= max_steps:
        step(t - dt, dt)
        diagnostics(t)
        t += dt
        n += 1
    return n - 1


def tick_due(t: float, start: float, dt: float, tick: float) -> bool:
    """examples/advection/include/application.h:464-471"""
    if t == start:
        return True
    return int((t + 0.00000000001 - start) / tick) != int((t + 0.00000000001 - start - dt) / tick)


def hyperrectangle_exact(dim: int) -> Func:
    """examples/advection/cases/hyperrectangle.h:29-66: sin(2 pi (x0 - a0 t)) prod cos(2 pi (x_d - a_d t)),
    a = (1, 0.15, -0.05, 0, ...)."""
    adv = [1.0, 0.15, -0.05] + [0.0] * 3
    return make_func(2, 1.0, omega=[2.0 * math.pi] * dim, speed=adv[:dim], phase=[0.0] * dim,
                     cosine=[0] + [1] * (dim - 1))


def run_hyperrectangle(dim_x: int, dim_v: int, degree: int, subdivisions: Sequence[int], periodic: bool,
                       collocation: bool, rk: str = "rk45", final_time: float = 1.0, time_step: float = 0.1,
                       cfl: float = 0.3, tick: float = 0.1, skew: float = 0.0) -> List[tuple]:
    """Runs the reference's advection application on the ``hyperrectangle`` case and returns the
    diagnostics rows (time, norm, error) that it prints."""
    dim = dim_x + dim_v
    exact = hyperrectangle_exact(dim)
    p = Problem(dim_x, dim_v, degree, cells=list(subdivisions), lo=[-1.0] * dim, hi=[1.0] * dim,
                velocity=[1.0, 0.15, -0.05, 0.0, 0.0, 0.0][:dim], periodic_x=periodic, periodic_v=periodic,
                collocation=collocation, skew=skew, bc_func=None if periodic else exact)
    sol = interpolate(p, exact, 0.0)
    dt = time_step_rule(time_step, cfl, critical_time_step(p), degree, 0.0, final_time)
    Ki = np.zeros_like(sol)
    Ti = np.zeros_like(sol)
    rows = []

    def step(t, h):
        lsrk_step(p, rk, sol, t, h, Ki, Ti)

    def diag(t):
        if tick_due(t, 0.0, dt, tick):
            n, e = norm_and_error(p, exact, t, sol)
            rows.append((t, n, e))

    time_loop(0.0, final_time, dt, step, diag)
    return rows


# --------------------------------------------------------------------------
# Vlasov-Poisson (examples/vlasov_poisson/include/application.h:400-700)
# --------------------------------------------------------------------------

def x_dofs(p: Problem) -> int:
    return int(np.prod(p.cells[:p.dim_x])) * (p.degree + 1) ** p.dim_x


def poisson_apply(p: Problem, u: np.ndarray) -> np.ndarray:
    out = np.empty_like(u)
    cp = p.c()
    _check(lib().hdo_poisson_apply(ctypes.byref(cp), _ptr(u), _ptr(out)), "poisson_apply")
    return out


def poisson_rhs(p: Problem, rho: np.ndarray) -> np.ndarray:
    out = np.empty_like(rho)
    cp = p.c()
    _check(lib().hdo_poisson_rhs(ctypes.byref(cp), _ptr(rho), _ptr(out)), "poisson_rhs")
    return out


def poisson_solve(p: Problem, rhs: np.ndarray, phi: np.ndarray, rel_tol: float = 1e-12, max_it: int = 100000) -> int:
    it = ctypes.c_int(0)
    cp = p.c()
    _check(lib().hdo_poisson_solve(ctypes.byref(cp), _ptr(rhs), _ptr(phi), rel_tol, max_it, ctypes.byref(it)),
           "poisson_solve")
    return it.value


def vp_field(p: Problem, phi: np.ndarray) -> np.ndarray:
    E = np.zeros(x_dofs(p) * p.dim_x)
    cp = p.c()
    _check(lib().hdo_vp_field(ctypes.byref(cp), _ptr(phi), _ptr(E)), "vp_field")
    return E


class VPState:
    """Potential and field carried between operator evaluations (the reference keeps
    `potential` as the CG initial guess and prints the energy of the last one)."""

    def __init__(self, p: Problem, cg_tol: float = 1e-12):
        self.p = p
        self.phi = np.zeros(x_dofs(p))
        self.E = np.zeros(x_dofs(p) * p.dim_x)
        self.cg_tol = cg_tol
        self.iterations = []

    def operator(self, src: np.ndarray, dst: np.ndarray, t: float) -> None:
        it = ctypes.c_int(0)
        cp = self.p.c()
        _check(lib().hdo_vp_operator(ctypes.byref(cp), _ptr(src), _ptr(dst), t, _ptr(self.phi), _ptr(self.E),
                                     self.cg_tol, ctypes.byref(it)), "vp_operator")
        self.iterations.append(it.value)

    def diagnostics(self, f: np.ndarray) -> np.ndarray:
        out = np.zeros(self.p.dim_x + 3 + self.p.dim_v)
        cp = self.p.c()
        _check(lib().hdo_vp_diagnostics(ctypes.byref(cp), _ptr(f), _ptr(self.phi), _ptr(out)), "vp_diagnostics")
        return out


def vp_initial_function(dim_x: int, dim_v: int, eps: float = 0.01, k: float = 0.5,
                        perturbed_dims: Sequence[int] = (0,)) -> Func:
    """(1 + eps prod_{d in perturbed_dims} cos(k x_d)) prod_v exp(-v^2/2)/sqrt(2 pi)
    (examples/vlasov_poisson/cases/hyperrectangle.h:45-58 perturbs x_0 only)."""
    cos_flags = [1 if d in perturbed_dims else 0 for d in range(dim_x)] + [2] * dim_v
    return make_func(3, eps, omega=[k] * dim_x + [0.0] * dim_v, cosine=cos_flags)


def run_vp_hyperrectangle(dim_x: int = 2, dim_v: int = 2, degree: int = 3, cells_x: int = 4, cells_v: int = 4,
                          collocation: bool = False, final_time: float = 0.5, time_step: float = 0.1,
                          cfl: float = 0.05, tick: float = 0.1, rk: str = "rk45", cg_tol: float = 1e-12):
    """The reference's Vlasov-Poisson application on its hyperrectangle case (x in [0, 4 pi]^dim_x,
    v in [-6, 6]^dim_v, periodic, transport direction (1, .., 6, ..) for the time-step rule);
    returns the diagnostics rows (time, energy components, mass, l2, kinetic energy, momentum)."""
    D = dim_x + dim_v
    p = Problem(dim_x, dim_v, degree, [cells_x] * dim_x + [cells_v] * dim_v, [0.0] * dim_x + [-6.0] * dim_v,
                [4 * math.pi] * dim_x + [6.0] * dim_v, [1.0] * dim_x + [6.0] * dim_v, collocation=collocation)
    f0 = vp_initial_function(dim_x, dim_v)
    sol = interpolate(p, f0, 0.0)
    dt = time_step_rule(time_step, cfl, critical_time_step(p), degree, 0.0, final_time)
    st = VPState(p, cg_tol)
    cp = p.c()
    st.p = p
    rows = []

    def step(t, h):
        lsrk_step_op(rk, sol, t, h, st.operator)

    def diag(t):
        if tick_due(t, 0.0, dt, tick):
            rows.append((t,) + tuple(st.diagnostics(sol)))

    time_loop(0.0, final_time, dt, step, diag)
    return rows, st
