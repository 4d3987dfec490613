"""The parity tests of the advection kernels with the bounds-checked library
(-DHD_CHECK: every global load and store of the ECL kernels checks its index and
records a violation in the device status, status 4, instead of accessing
memory), plus a sweep that asserts status 0 after launches of every generic
kernel shape (FP64 storage in both arithmetics).  Building the checked library takes minutes, so this runs only
when HYPERDEAL_GB300_RUN_CHECK_BUILD=1 is set:

    HYPERDEAL_GB300_RUN_CHECK_BUILD=1 python -m pytest tests/test_gpu_check_build.py -m gpu
"""
import os
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(os.environ.get("HYPERDEAL_GB300_RUN_CHECK_BUILD") != "1",
                                 reason="set HYPERDEAL_GB300_RUN_CHECK_BUILD=1 to build and run the checked library")]

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SWEEP = r'''
import itertools, numpy as np, torch
from hyperdeal_gb300 import _lib, advection as A, partition as Pt
assert _lib.lib_path().endswith("_check.so")
bad = []
for dx, dv in itertools.product((1, 2, 3), (1, 2, 3)):
    for k in (1, 2, 3, 4, 5):
        D = dx + dv
        if (k + 1) ** D > 4096 * 2:
            continue
        cells = [2] * D
        for dtype in ("f64", "f32"):
            p = A.AdvectionParameters(dx, dv, k, cells[:dx], cells[dx:], [0] * dx, [1] * dx, [0] * dv, [1] * dv,
                                      [0.9 - 0.3 * d for d in range(D)], dtype=dtype)
            try:
                op = A.AdvectionOperation(p)
            except A.HdError:
                continue
            for arith in (("native", "fp32x2") if dtype == "f64" else ("native",)):
                op.set_arithmetic(arith)
                u = torch.randn(op.n_dofs, dtype=op.dtype, device="cuda")
                it = A.LowStorageRungeKuttaIntegrator(op.initialize_dof_vector(), op.initialize_dof_vector(), "rk45")
                it.perform_time_step(u, 0.0, 1e-3, op)
                if op.device_status() != 0:
                    bad.append((dx, dv, k, dtype, arith))
# the pipelined kernel's 4D units (16 cells along x0), both velocity signs
for vel in ([0.9, 0.7, 0.5, 0.3], [-0.9, 0.7, -0.5, 0.3]):
    p = A.AdvectionParameters(2, 2, 3, [16, 2], [2, 3], [0] * 2, [1] * 2, [0] * 2, [1] * 2, vel, dtype="f32")
    op = A.AdvectionOperation(p)
    assert op.kernel == "pipelined"
    u = torch.randn(op.n_dofs, dtype=op.dtype, device="cuda")
    it = A.LowStorageRungeKuttaIntegrator(op.initialize_dof_vector(), op.initialize_dof_vector(), "rk45")
    it.perform_time_step(u, 0.0, 1e-3, op)
    if op.device_status() != 0:
        bad.append(("pipelined 4D", vel))
g = Pt.LocalPartGroup(A.AdvectionParameters(3, 3, 3, [2] * 3, [2, 2, 4], [0] * 3, [1] * 3, [0] * 3, [1] * 3,
                                            [1, .8, .6, .4, .3, .2], dtype="f32"), 2)
sols = g.initialize_dof_vectors()
its = [A.LowStorageRungeKuttaIntegrator(o.initialize_dof_vector(), o.initialize_dof_vector()) for o in g.ops]
g.perform_time_step(its, sols, 0.0, 1e-3)
bad += [("part", o.part) for o in g.ops if o.device_status() != 0]
assert not bad, bad
print("sweep ok")
'''


def _env():
    env = dict(os.environ, HYPERDEAL_GB300_CHECK="1")
    env.pop("HYPERDEAL_GB300_RUN_CHECK_BUILD", None)
    return env


def test_checked_library_builds():
    from hyperdeal_gb300 import build as B
    path = B.build(check=True)
    assert path.endswith("_check.so") and os.path.exists(path)


def test_no_bounds_violation_in_the_kernel_sweep():
    r = subprocess.run([sys.executable, "-c", SWEEP], cwd=ROOT, env=_env(), capture_output=True, text=True,
                       timeout=1800)
    assert r.returncode == 0 and "sweep ok" in r.stdout, r.stdout[-2000:] + r.stderr[-3000:]


def test_parity_suite_passes_with_the_checked_library():
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-m", "gpu", "tests/test_gpu_parity.py",
                        "tests/test_gpu_partition.py", "tests/test_gpu_fp32x2.py", "tests/test_gpu_layout.py",
                        "tests/test_gpu_pipelined4d.py"],
                       cwd=ROOT, env=_env(), capture_output=True, text=True, timeout=3600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
