"""Race canary for the fused LSRK step (planted in the oracle, on the CPU).

The fused stage kernel reads the upwind neighbours' faces of the stage input T
while it writes the next stage input, so it must not write T in place: the
three vectors rotate roles (hd_lsrk_step).  This test restates the fused step
cell by cell on the oracle, once with the rotation (the next input written to
a separate vector) and once without it (written over T while later cells still
read T -- what a missing rotation would do), and shows that the comparison the
GPU tests make between the fused and the unfused step (1e-12 in FP64,
tests/test_gpu_parity.py) catches the missing rotation by many orders of
magnitude, while the rotated restatement passes it.
"""
import math

import numpy as np

from oracle import oracle as O


def fused_step_cellwise(prob, u, t, dt, rotate):
    a, b = O.lsrk_coefficients("rk45")
    ns = len(b)
    c = [0.0] * ns
    sb = 0.0
    for s in range(1, ns):
        c[s] = sb + a[s - 1]
        sb += b[s - 1]
    NC = (prob.degree + 1) ** prob.dim
    ncells = prob.n_dofs // NC
    U = u.copy()
    T = u.copy()
    for s in range(ns):
        Tn = np.empty_like(T) if rotate else T
        fa = a[s] * dt if s < ns - 1 else 0.0
        for cell in range(ncells):  # increasing ids: the upwind neighbours come first
            K = O.apply_cells(prob, T, np.array([cell]), t + c[s] * dt)
            sl = slice(cell * NC, (cell + 1) * NC)
            u_old = U[sl].copy()
            U[sl] = u_old + b[s] * dt * K
            Tn[sl] = u_old + fa * K
        T = Tn
    return U


def test_missing_rotation_is_caught_by_the_fused_vs_unfused_comparison():
    prob = O.Problem(1, 1, 3, [6, 5], [0.0, 0.0], [1.0, 1.0], [1.0, 0.5])
    f = O.make_func(2, 1.0, omega=[2 * math.pi] * 2, speed=[0.0, 0.0])
    u = O.interpolate(prob, f)
    dt = 0.2 * O.critical_time_step(prob) / 3 ** 1.5
    ref = u.copy()
    O.lsrk_step(prob, "rk45", ref, 0.0, dt)
    scale = np.abs(ref).max()
    good = fused_step_cellwise(prob, u, 0.0, dt, rotate=True)
    bad = fused_step_cellwise(prob, u, 0.0, dt, rotate=False)
    assert np.abs(good - ref).max() / scale < 1e-13
    assert np.abs(bad - ref).max() / scale > 1e-4
